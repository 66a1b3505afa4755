// rt_assets.cpp — host-side asset decoding declared in include/rtassets.h:
// a PNG decoder producing the reference's RGBA8 texels and a glTF-binary
// (GLB) model reader producing its vertex / index arrays and image order.
//
// Reference behaviour restated (paths inside the reference project):
//   load_png_image_from_bytes      src/util_functions.rs:239-265
//   Model::load_gltf               src/util_structs.rs:1049-1156
//   load_images_from_material      src/util_structs.rs:982-1024
//   load_image_from_gltf_texture   src/util_structs.rs:934-980
// The reference does this with the `image 0.23.14` / `png 0.16.8` and
// `gltf 0.16.0` crates; the formats are restated here from their published
// specifications (RFC 1950 zlib, RFC 1951 DEFLATE, PNG 2nd edition, glTF 2.0).
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "rt_error.h"
#include "rtassets.h"

namespace {

// An asset that cannot be decoded: status code plus message.
struct AssetError {
    int32_t code;
    std::string msg;
};

[[noreturn]] void bad(int32_t code, const char* fmt, ...) {
    char buf[400];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw AssetError{code, buf};
}

uint32_t be32(const uint8_t* p) {
    return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3];
}
uint32_t le32(const uint8_t* p) {
    return (uint32_t)p[3] << 24 | (uint32_t)p[2] << 16 | (uint32_t)p[1] << 8 | p[0];
}
uint16_t le16(const uint8_t* p) { return (uint16_t)(p[0] | p[1] << 8); }
float lef32(const uint8_t* p) {
    uint32_t u = le32(p);
    float f;
    memcpy(&f, &u, 4);
    return f;
}

// ---------------------------------------------------------------------------
// Checksums: CRC-32 (ISO 3309, reflected polynomial 0xEDB88320) over PNG
// chunks, Adler-32 (RFC 1950) over the zlib payload.
// ---------------------------------------------------------------------------
struct Crc32Table {
    uint32_t t[256];
    Crc32Table() {
        for (uint32_t i = 0; i < 256; i++) {
            uint32_t c = i;
            for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
    }
};
const Crc32Table kCrc;

uint32_t crc32(const uint8_t* p, size_t n) {
    uint32_t c = 0xFFFFFFFFu;
    for (size_t i = 0; i < n; i++) c = kCrc.t[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return c ^ 0xFFFFFFFFu;
}

uint32_t adler32(const uint8_t* p, size_t n) {
    uint32_t a = 1, b = 0;
    while (n) {
        size_t k = n < 5552 ? n : 5552;   // largest run before b can exceed 2^32
        n -= k;
        while (k--) {
            a += *p++;
            b += a;
        }
        a %= 65521;
        b %= 65521;
    }
    return b << 16 | a;
}

// ---------------------------------------------------------------------------
// DEFLATE (RFC 1951).  Bits are read LSB-first; Huffman codes are matched
// through a 10-bit lookup table, longer codes by walking the canonical code
// one bit at a time.
// ---------------------------------------------------------------------------
class BitReader {
public:
    BitReader(const uint8_t* p, size_t n) : p_(p), end_(p + n) {}

    void refill() {
        while (cnt_ <= 56) {
            uint64_t b = 0;
            if (p_ < end_) b = *p_++;
            else if (++past_end_ > 8) bad(RT_ERR_INVALID, "deflate stream is truncated");
            buf_ |= b << cnt_;
            cnt_ += 8;
        }
    }
    uint32_t peek(int n) const { return (uint32_t)(buf_ & ((1ull << n) - 1)); }
    void drop(int n) {
        buf_ >>= n;
        cnt_ -= n;
    }
    uint32_t bits(int n) {  // n <= 32
        if (cnt_ < n) refill();
        uint32_t v = peek(n);
        drop(n);
        return v;
    }
    void align_byte() { drop(cnt_ & 7); }
    // Bytes consumed so far (after align_byte), with truncation detected.
    size_t consumed(size_t total) const {
        size_t fed = total - (size_t)(end_ - p_) + past_end_;
        size_t used = fed - (size_t)(cnt_ / 8);
        if (used > total) bad(RT_ERR_INVALID, "deflate stream is truncated");
        return used;
    }
    int available() const { return cnt_; }

private:
    const uint8_t* p_;
    const uint8_t* end_;
    uint64_t buf_ = 0;
    int cnt_ = 0;
    int past_end_ = 0;
};

uint32_t reverse_bits(uint32_t v, int n) {
    uint32_t r = 0;
    for (int i = 0; i < n; i++) r |= ((v >> i) & 1) << (n - 1 - i);
    return r;
}

// Canonical Huffman decoding as RFC 1951 section 3.2.2 defines the codes
// (codes of each length are consecutive integers, assigned in symbol order):
// the slow path walks the lengths 1..15 keeping the first code and the first
// symbol index of each length (the counting decode that zlib's
// contrib/puff/puff.c also uses), and a kFast-bit table indexed by the
// bit-reversed next bits resolves the short codes in one lookup.
class Huffman {
public:
    static constexpr int kFast = 10;

    // lengths[i] = code length of symbol i (0 = unused).  Over-subscribed sets
    // are rejected; incomplete sets are allowed (an unassigned code is an
    // error when it is met).
    void build(const uint8_t* lengths, int n) {
        memset(count_, 0, sizeof count_);
        for (int i = 0; i < n; i++) count_[lengths[i]]++;
        count_[0] = 0;
        int left = 1;
        for (int len = 1; len <= 15; len++) {
            left <<= 1;
            left -= count_[len];
            if (left < 0) bad(RT_ERR_INVALID, "deflate: over-subscribed Huffman code");
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int len = 1; len < 15; len++) offs[len + 1] = (uint16_t)(offs[len] + count_[len]);
        for (int i = 0; i < n; i++)
            if (lengths[i]) symbols_[offs[lengths[i]]++] = (uint16_t)i;
        // canonical codes: shorter codes first, symbols in order within a length
        memset(fast_, 0, sizeof fast_);
        uint32_t code = 0;
        int k = 0;
        for (int len = 1; len <= 15; len++) {
            for (int j = 0; j < count_[len]; j++, k++, code++) {
                if (len > kFast) continue;
                uint32_t r = reverse_bits(code, len);
                for (uint32_t f = r; f < (1u << kFast); f += 1u << len)
                    fast_[f] = (uint16_t)(symbols_[k] << 4 | len);
            }
            code <<= 1;
        }
    }

    int decode(BitReader& br) const {
        if (br.available() < 16) br.refill();
        uint16_t e = fast_[br.peek(kFast)];
        if (e & 15) {
            br.drop(e & 15);
            return e >> 4;
        }
        int code = 0, first = 0, index = 0;
        for (int len = 1; len <= 15; len++) {
            code |= (int)br.bits(1);
            int c = count_[len];
            if (code - first < c) return symbols_[index + code - first];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        bad(RT_ERR_INVALID, "deflate: invalid Huffman code");
    }

private:
    uint16_t count_[16];
    uint16_t symbols_[320];
    uint16_t fast_[1 << kFast];
};

// RFC 1951 section 3.2.5: base values and extra bits of length codes 257..285
// and distance codes 0..29.
const uint16_t kLenBase[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1,   2,   3,   4,   5,   7,    9,    13,   17,   25,   33,   49,   65,    97,    129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};
// order in which code-length code lengths are stored (section 3.2.7)
const uint8_t kClenOrder[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};

// Inflates a raw DEFLATE stream into out[0, cap); returns bytes written.
size_t inflate_raw(BitReader& br, uint8_t* out, size_t cap) {
    size_t pos = 0;
    Huffman lit, dist;
    bool last = false;
    while (!last) {
        last = br.bits(1) != 0;
        uint32_t type = br.bits(2);
        if (type == 0) {  // stored
            br.align_byte();
            uint32_t len = br.bits(16), nlen = br.bits(16);
            if ((len ^ 0xFFFFu) != nlen) bad(RT_ERR_INVALID, "deflate: stored block length check failed");
            if (len > cap - pos) bad(RT_ERR_INVALID, "deflate: data exceeds the image size");
            for (uint32_t i = 0; i < len; i++) out[pos++] = (uint8_t)br.bits(8);
            continue;
        }
        if (type == 3) bad(RT_ERR_INVALID, "deflate: reserved block type");
        uint8_t lengths[320];
        int hlit, hdist;
        if (type == 1) {  // fixed codes (section 3.2.6)
            hlit = 288;
            hdist = 30;
            for (int i = 0; i < 144; i++) lengths[i] = 8;
            for (int i = 144; i < 256; i++) lengths[i] = 9;
            for (int i = 256; i < 280; i++) lengths[i] = 7;
            for (int i = 280; i < 288; i++) lengths[i] = 8;
            for (int i = 0; i < 30; i++) lengths[288 + i] = 5;
        } else {  // dynamic codes (section 3.2.7)
            hlit = (int)br.bits(5) + 257;
            hdist = (int)br.bits(5) + 1;
            int hclen = (int)br.bits(4) + 4;
            if (hlit > 286 || hdist > 30) bad(RT_ERR_INVALID, "deflate: too many length or distance codes");
            uint8_t cl[19] = {0};
            for (int i = 0; i < hclen; i++) cl[kClenOrder[i]] = (uint8_t)br.bits(3);
            Huffman clh;
            clh.build(cl, 19);
            int n = 0;
            while (n < hlit + hdist) {
                int sym = clh.decode(br);
                if (sym < 16) {
                    lengths[n++] = (uint8_t)sym;
                    continue;
                }
                int rep;
                uint8_t val = 0;
                if (sym == 16) {
                    if (n == 0) bad(RT_ERR_INVALID, "deflate: repeat with no previous length");
                    val = lengths[n - 1];
                    rep = 3 + (int)br.bits(2);
                } else if (sym == 17) {
                    rep = 3 + (int)br.bits(3);
                } else {
                    rep = 11 + (int)br.bits(7);
                }
                if (n + rep > hlit + hdist) bad(RT_ERR_INVALID, "deflate: code lengths overflow");
                while (rep--) lengths[n++] = val;
            }
            if (lengths[256] == 0) bad(RT_ERR_INVALID, "deflate: no end-of-block code");
            // distance lengths follow the literal/length ones
            memmove(lengths + 288, lengths + hlit, (size_t)hdist);
            for (int i = hlit; i < 288; i++) lengths[i] = 0;
            hlit = 288;
        }
        lit.build(lengths, hlit);
        dist.build(lengths + 288, hdist);
        for (;;) {
            int sym = lit.decode(br);
            if (sym < 256) {
                if (pos == cap) bad(RT_ERR_INVALID, "deflate: data exceeds the image size");
                out[pos++] = (uint8_t)sym;
                continue;
            }
            if (sym == 256) break;
            sym -= 257;
            if (sym >= 29) bad(RT_ERR_INVALID, "deflate: invalid length code");
            size_t len = kLenBase[sym] + br.bits(kLenExtra[sym]);
            int ds = dist.decode(br);
            if (ds >= 30) bad(RT_ERR_INVALID, "deflate: invalid distance code");
            size_t d = kDistBase[ds] + br.bits(kDistExtra[ds]);
            if (d > pos) bad(RT_ERR_INVALID, "deflate: distance before the start of the data");
            if (len > cap - pos) bad(RT_ERR_INVALID, "deflate: data exceeds the image size");
            const uint8_t* src = out + pos - d;
            uint8_t* dst = out + pos;
            for (size_t i = 0; i < len; i++) dst[i] = src[i];   // overlapping copies repeat the run
            pos += len;
        }
    }
    return pos;
}

// zlib stream (RFC 1950) holding exactly `expect` bytes.
void zlib_inflate(const uint8_t* p, size_t n, uint8_t* out, size_t expect) {
    if (n < 6) bad(RT_ERR_INVALID, "zlib stream too short");
    uint32_t cmf = p[0], flg = p[1];
    if ((cmf & 15) != 8 || (cmf >> 4) > 7) bad(RT_ERR_INVALID, "zlib: not a deflate stream");
    if ((cmf << 8 | flg) % 31 != 0) bad(RT_ERR_INVALID, "zlib: header check failed");
    if (flg & 0x20) bad(RT_ERR_UNSUPPORTED, "zlib: preset dictionary");
    BitReader br(p + 2, n - 2);
    size_t got = inflate_raw(br, out, expect);
    if (got != expect) bad(RT_ERR_INVALID, "PNG image data holds %zu bytes, %zu expected", got, expect);
    br.align_byte();
    size_t used = 2 + br.consumed(n - 2);
    if (used + 4 > n) bad(RT_ERR_INVALID, "zlib: missing Adler-32");
    if (be32(p + used) != adler32(out, expect)) bad(RT_ERR_INVALID, "zlib: Adler-32 mismatch");
}

// ---------------------------------------------------------------------------
// PNG (ISO/IEC 15948, PNG 2nd edition).
// ---------------------------------------------------------------------------
struct Png {
    uint32_t width = 0, height = 0;
    uint8_t depth = 0, color = 0, interlace = 0;
    std::vector<uint8_t> palette;   // RGB triples
    std::vector<uint8_t> trns;      // raw tRNS chunk
    std::vector<uint8_t> idat;
};

int png_channels(uint8_t color) {
    switch (color) {
        case 0: return 1;
        case 2: return 3;
        case 3: return 1;
        case 4: return 2;
        case 6: return 4;
    }
    return 0;
}

bool png_depth_ok(uint8_t color, uint8_t depth) {
    switch (color) {
        case 0: return depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16;
        case 3: return depth == 1 || depth == 2 || depth == 4 || depth == 8;
        case 2: case 4: case 6: return depth == 8 || depth == 16;
    }
    return false;
}

const uint8_t kPngSignature[8] = {137, 80, 78, 71, 13, 10, 26, 10};
constexpr uint64_t kMaxPixels = 1ull << 28;

// Reads the chunk stream; with header_only, stops after IHDR.
Png png_parse(const uint8_t* p, size_t n, bool header_only) {
    if (n < 8 || memcmp(p, kPngSignature, 8) != 0) bad(RT_ERR_INVALID, "not a PNG file");
    Png png;
    size_t at = 8;
    bool have_header = false, have_end = false;
    while (at < n) {
        if (n - at < 12) bad(RT_ERR_INVALID, "PNG chunk header truncated");
        uint32_t len = be32(p + at);
        const uint8_t* type = p + at + 4;
        if (len > n - at - 12) bad(RT_ERR_INVALID, "PNG chunk '%.4s' truncated", (const char*)type);
        const uint8_t* data = type + 4;
        if (be32(data + len) != crc32(type, (size_t)len + 4))
            bad(RT_ERR_INVALID, "PNG chunk '%.4s' CRC mismatch", (const char*)type);
        at += 12 + (size_t)len;
        if (!have_header && memcmp(type, "IHDR", 4) != 0) bad(RT_ERR_INVALID, "PNG does not start with IHDR");
        if (memcmp(type, "IHDR", 4) == 0) {
            if (have_header || len != 13) bad(RT_ERR_INVALID, "bad PNG IHDR");
            png.width = be32(data);
            png.height = be32(data + 4);
            png.depth = data[8];
            png.color = data[9];
            png.interlace = data[12];
            if (png.width == 0 || png.height == 0 || png.width > (1u << 24) || png.height > (1u << 24) ||
                (uint64_t)png.width * png.height > kMaxPixels)
                bad(RT_ERR_TOO_LARGE, "PNG size %ux%u is not supported", png.width, png.height);
            if (!png_depth_ok(png.color, png.depth))
                bad(RT_ERR_INVALID, "PNG colour type %u with bit depth %u", png.color, png.depth);
            if (data[10] != 0 || data[11] != 0 || png.interlace > 1)
                bad(RT_ERR_INVALID, "PNG compression / filter / interlace method not defined");
            have_header = true;
            if (header_only) return png;
        } else if (memcmp(type, "PLTE", 4) == 0) {
            if (len == 0 || len % 3 != 0 || len > 768) bad(RT_ERR_INVALID, "bad PNG palette");
            png.palette.assign(data, data + len);
        } else if (memcmp(type, "tRNS", 4) == 0) {
            png.trns.assign(data, data + len);
        } else if (memcmp(type, "IDAT", 4) == 0) {
            png.idat.insert(png.idat.end(), data, data + len);
        } else if (memcmp(type, "IEND", 4) == 0) {
            have_end = true;
            break;
        } else if (!(type[0] & 0x20)) {
            bad(RT_ERR_UNSUPPORTED, "unknown critical PNG chunk '%.4s'", (const char*)type);
        }  // other ancillary chunks (gAMA, iCCP, pHYs, text ...) do not change the texels
    }
    if (!have_end) bad(RT_ERR_INVALID, "PNG has no IEND chunk");
    if (png.color == 3 && png.palette.empty()) bad(RT_ERR_INVALID, "PNG palette image without PLTE");
    if (png.idat.empty()) bad(RT_ERR_INVALID, "PNG has no image data");
    if (png.color == 0 && !png.trns.empty() && png.trns.size() != 2) bad(RT_ERR_INVALID, "bad PNG tRNS");
    if (png.color == 2 && !png.trns.empty() && png.trns.size() != 6) bad(RT_ERR_INVALID, "bad PNG tRNS");
    if (png.color == 3 && png.trns.size() > png.palette.size() / 3) bad(RT_ERR_INVALID, "bad PNG tRNS");
    if ((png.color == 4 || png.color == 6) && !png.trns.empty()) bad(RT_ERR_INVALID, "tRNS with an alpha channel");
    return png;
}

// Adam7 passes: first column / row and steps.
struct Pass {
    uint32_t x0, y0, dx, dy;
};
const Pass kAdam7[7] = {{0, 0, 8, 8}, {4, 0, 8, 8}, {0, 4, 4, 8}, {2, 0, 4, 4},
                        {0, 2, 2, 4}, {1, 0, 2, 2}, {0, 1, 1, 2}};
const Pass kWhole = {0, 0, 1, 1};

uint32_t pass_extent(uint32_t size, uint32_t start, uint32_t step) {
    return size > start ? (size - start + step - 1) / step : 0;
}

uint8_t paeth(int a, int b, int c) {
    int p = a + b - c;
    int pa = p > a ? p - a : a - p;
    int pb = p > b ? p - b : b - p;
    int pc = p > c ? p - c : c - p;
    if (pa <= pb && pa <= pc) return (uint8_t)a;
    return (uint8_t)(pb <= pc ? b : c);
}

// Reverses the per-row filters of one pass in place (section 9).
void unfilter(uint8_t* rows, uint32_t h, size_t rowbytes, size_t bpp) {
    uint8_t* prev = nullptr;
    for (uint32_t y = 0; y < h; y++) {
        uint8_t* f = rows + (size_t)y * (rowbytes + 1);
        uint8_t* r = f + 1;
        switch (f[0]) {
            case 0: break;
            case 1:
                for (size_t i = bpp; i < rowbytes; i++) r[i] = (uint8_t)(r[i] + r[i - bpp]);
                break;
            case 2:
                if (prev)
                    for (size_t i = 0; i < rowbytes; i++) r[i] = (uint8_t)(r[i] + prev[i]);
                break;
            case 3:
                for (size_t i = 0; i < rowbytes; i++) {
                    int a = i >= bpp ? r[i - bpp] : 0, b = prev ? prev[i] : 0;
                    r[i] = (uint8_t)(r[i] + ((a + b) >> 1));
                }
                break;
            case 4:
                for (size_t i = 0; i < rowbytes; i++) {
                    int a = i >= bpp ? r[i - bpp] : 0, b = prev ? prev[i] : 0;
                    int c = (prev && i >= bpp) ? prev[i - bpp] : 0;
                    r[i] = (uint8_t)(r[i] + paeth(a, b, c));
                }
                break;
            default: bad(RT_ERR_INVALID, "PNG row filter type %u", f[0]);
        }
        prev = r;
    }
}

// 16-bit channel to 8 bits: the high byte (the `image` 0.23 crate's
// conversion behind to_rgba8).
inline uint8_t down16(uint32_t v) { return (uint8_t)(v >> 8); }

// Writes the RGBA8 texels of one pass's unfiltered rows into out.
void expand_pass(const Png& png, const uint8_t* rows, const Pass& ps, uint32_t pw, uint32_t ph, size_t rowbytes,
                 uint8_t* out) {
    const int ch = png_channels(png.color);
    const uint32_t d = png.depth;
    const uint32_t maxv = (1u << d) - 1;
    const bool key = !png.trns.empty();
    const uint32_t kg = key && png.color == 0 ? (uint32_t)png.trns[0] << 8 | png.trns[1] : 0;
    uint32_t kr = 0, kgr = 0, kb = 0;
    if (key && png.color == 2) {
        kr = (uint32_t)png.trns[0] << 8 | png.trns[1];
        kgr = (uint32_t)png.trns[2] << 8 | png.trns[3];
        kb = (uint32_t)png.trns[4] << 8 | png.trns[5];
    }
    for (uint32_t j = 0; j < ph; j++) {
        const uint8_t* r = rows + (size_t)j * (rowbytes + 1) + 1;
        uint8_t* orow = out + ((size_t)(ps.y0 + j * ps.dy) * png.width) * 4;
        for (uint32_t i = 0; i < pw; i++) {
            uint8_t* o = orow + (size_t)(ps.x0 + i * ps.dx) * 4;
            // raw samples of pixel i
            uint32_t s[4] = {0, 0, 0, 0};
            if (d < 8) {
                size_t bit = (size_t)i * d;
                s[0] = (r[bit >> 3] >> (8 - d - (bit & 7))) & maxv;
            } else if (d == 8) {
                for (int c = 0; c < ch; c++) s[c] = r[(size_t)i * ch + c];
            } else {
                for (int c = 0; c < ch; c++) s[c] = (uint32_t)r[((size_t)i * ch + c) * 2] << 8 | r[((size_t)i * ch + c) * 2 + 1];
            }
            auto to8 = [&](uint32_t v) -> uint8_t {
                if (d == 16) return down16(v);
                if (d == 8) return (uint8_t)v;
                return (uint8_t)(v * (255 / maxv));
            };
            switch (png.color) {
                case 0: {
                    uint8_t g = to8(s[0]);
                    o[0] = o[1] = o[2] = g;
                    o[3] = key && s[0] == kg ? 0 : 255;
                    break;
                }
                case 2:
                    o[0] = to8(s[0]);
                    o[1] = to8(s[1]);
                    o[2] = to8(s[2]);
                    o[3] = key && s[0] == kr && s[1] == kgr && s[2] == kb ? 0 : 255;
                    break;
                case 3: {
                    uint32_t idx = s[0];
                    if (idx * 3 >= png.palette.size()) bad(RT_ERR_INVALID, "PNG palette index %u out of range", idx);
                    o[0] = png.palette[idx * 3];
                    o[1] = png.palette[idx * 3 + 1];
                    o[2] = png.palette[idx * 3 + 2];
                    o[3] = idx < png.trns.size() ? png.trns[idx] : 255;
                    break;
                }
                case 4: {
                    uint8_t g = to8(s[0]);
                    o[0] = o[1] = o[2] = g;
                    o[3] = to8(s[1]);
                    break;
                }
                default:
                    o[0] = to8(s[0]);
                    o[1] = to8(s[1]);
                    o[2] = to8(s[2]);
                    o[3] = to8(s[3]);
            }
        }
    }
}

void png_decode(const uint8_t* p, size_t n, std::vector<uint8_t>& out, uint32_t& w, uint32_t& h) {
    Png png = png_parse(p, n, false);
    w = png.width;
    h = png.height;
    const size_t bits_pp = (size_t)png_channels(png.color) * png.depth;
    const size_t bpp = bits_pp >= 8 ? bits_pp / 8 : 1;
    const Pass* passes = png.interlace ? kAdam7 : &kWhole;
    const int npass = png.interlace ? 7 : 1;
    size_t total = 0;
    for (int k = 0; k < npass; k++) {
        uint32_t pw = pass_extent(w, passes[k].x0, passes[k].dx), ph = pass_extent(h, passes[k].y0, passes[k].dy);
        if (pw && ph) total += (size_t)ph * ((pw * bits_pp + 7) / 8 + 1);
    }
    std::vector<uint8_t> raw(total);
    zlib_inflate(png.idat.data(), png.idat.size(), raw.data(), total);
    out.assign((size_t)w * h * 4, 0);
    size_t at = 0;
    for (int k = 0; k < npass; k++) {
        uint32_t pw = pass_extent(w, passes[k].x0, passes[k].dx), ph = pass_extent(h, passes[k].y0, passes[k].dy);
        if (!pw || !ph) continue;
        size_t rowbytes = (pw * bits_pp + 7) / 8;
        unfilter(raw.data() + at, ph, rowbytes, bpp);
        expand_pass(png, raw.data() + at, passes[k], pw, ph, rowbytes, out.data());
        at += (size_t)ph * (rowbytes + 1);
    }
}

// ---------------------------------------------------------------------------
// JSON (RFC 8259), enough of it for a glTF document: a tree of values.
// ---------------------------------------------------------------------------
struct Json {
    enum Kind { Null, Bool, Num, Str, Arr, Obj } kind = Null;
    bool b = false;
    double num = 0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    const Json* get(const char* key) const {
        if (kind != Obj) return nullptr;
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
};

class JsonParser {
public:
    JsonParser(const char* p, size_t n) : p_(p), end_(p + n) {}

    Json parse() {
        Json v = value(0);
        ws();
        if (p_ != end_) fail("trailing characters");
        return v;
    }

private:
    [[noreturn]] void fail(const char* what) { bad(RT_ERR_INVALID, "glTF JSON: %s", what); }
    void ws() {
        while (p_ < end_ && (*p_ == ' ' || *p_ == '\t' || *p_ == '\n' || *p_ == '\r')) p_++;
    }
    bool lit(const char* s) {
        size_t k = strlen(s);
        if ((size_t)(end_ - p_) >= k && memcmp(p_, s, k) == 0) {
            p_ += k;
            return true;
        }
        return false;
    }
    static void put_utf8(std::string& s, uint32_t c) {
        if (c < 0x80) {
            s += (char)c;
        } else if (c < 0x800) {
            s += (char)(0xC0 | c >> 6);
            s += (char)(0x80 | (c & 63));
        } else if (c < 0x10000) {
            s += (char)(0xE0 | c >> 12);
            s += (char)(0x80 | (c >> 6 & 63));
            s += (char)(0x80 | (c & 63));
        } else {
            s += (char)(0xF0 | c >> 18);
            s += (char)(0x80 | (c >> 12 & 63));
            s += (char)(0x80 | (c >> 6 & 63));
            s += (char)(0x80 | (c & 63));
        }
    }
    uint32_t hex4() {
        if (end_ - p_ < 4) fail("bad \\u escape");
        uint32_t v = 0;
        for (int i = 0; i < 4; i++) {
            char c = *p_++;
            v <<= 4;
            if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
            else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
            else fail("bad \\u escape");
        }
        return v;
    }
    std::string string() {
        p_++;  // opening quote
        std::string s;
        for (;;) {
            if (p_ >= end_) fail("unterminated string");
            char c = *p_++;
            if (c == '"') return s;
            if ((unsigned char)c < 0x20) fail("control character in string");
            if (c != '\\') {
                s += c;
                continue;
            }
            if (p_ >= end_) fail("unterminated string");
            char e = *p_++;
            switch (e) {
                case '"': s += '"'; break;
                case '\\': s += '\\'; break;
                case '/': s += '/'; break;
                case 'b': s += '\b'; break;
                case 'f': s += '\f'; break;
                case 'n': s += '\n'; break;
                case 'r': s += '\r'; break;
                case 't': s += '\t'; break;
                case 'u': {
                    uint32_t c1 = hex4();
                    if (c1 >= 0xD800 && c1 < 0xDC00 && end_ - p_ >= 6 && p_[0] == '\\' && p_[1] == 'u') {
                        p_ += 2;
                        uint32_t c2 = hex4();
                        if (c2 < 0xDC00 || c2 >= 0xE000) fail("bad surrogate pair");
                        c1 = 0x10000 + ((c1 - 0xD800) << 10) + (c2 - 0xDC00);
                    }
                    put_utf8(s, c1);
                    break;
                }
                default: fail("bad escape");
            }
        }
    }
    double number() {
        const char* s = p_;
        if (p_ < end_ && *p_ == '-') p_++;
        auto digits = [&] {
            const char* d = p_;
            while (p_ < end_ && *p_ >= '0' && *p_ <= '9') p_++;
            if (p_ == d) fail("bad number");
        };
        digits();
        if (p_ < end_ && *p_ == '.') {
            p_++;
            digits();
        }
        if (p_ < end_ && (*p_ == 'e' || *p_ == 'E')) {
            p_++;
            if (p_ < end_ && (*p_ == '+' || *p_ == '-')) p_++;
            digits();
        }
        std::string t(s, p_);
        return strtod(t.c_str(), nullptr);
    }
    Json value(int depth) {
        if (depth > 64) fail("nesting too deep");
        ws();
        if (p_ >= end_) fail("unexpected end");
        Json v;
        char c = *p_;
        if (c == '{') {
            v.kind = Json::Obj;
            p_++;
            ws();
            if (p_ < end_ && *p_ == '}') {
                p_++;
                return v;
            }
            for (;;) {
                ws();
                if (p_ >= end_ || *p_ != '"') fail("expected a key");
                std::string k = string();
                ws();
                if (p_ >= end_ || *p_ != ':') fail("expected ':'");
                p_++;
                v.obj.emplace_back(std::move(k), value(depth + 1));
                ws();
                if (p_ < end_ && *p_ == ',') {
                    p_++;
                    continue;
                }
                if (p_ < end_ && *p_ == '}') {
                    p_++;
                    return v;
                }
                fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.kind = Json::Arr;
            p_++;
            ws();
            if (p_ < end_ && *p_ == ']') {
                p_++;
                return v;
            }
            for (;;) {
                v.arr.push_back(value(depth + 1));
                ws();
                if (p_ < end_ && *p_ == ',') {
                    p_++;
                    continue;
                }
                if (p_ < end_ && *p_ == ']') {
                    p_++;
                    return v;
                }
                fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.kind = Json::Str;
            v.str = string();
            return v;
        }
        if (lit("true")) {
            v.kind = Json::Bool;
            v.b = true;
            return v;
        }
        if (lit("false")) {
            v.kind = Json::Bool;
            return v;
        }
        if (lit("null")) return v;
        v.kind = Json::Num;
        v.num = number();
        return v;
    }

    const char* p_;
    const char* end_;
};

// ---------------------------------------------------------------------------
// glTF 2.0 binary container.
// ---------------------------------------------------------------------------
constexpr uint32_t kGlbMagic = 0x46546C67u;   // "glTF"
constexpr uint32_t kChunkJson = 0x4E4F534Au;  // "JSON"
constexpr uint32_t kChunkBin = 0x004E4942u;   // "BIN\0"
constexpr int kGlNearest = 9728;              // sampler magFilter NEAREST

struct Image {
    uint32_t width = 1, height = 1, format = 0, filter = RT_FILTER_NEAREST;
    std::shared_ptr<const std::vector<uint8_t>> texels;
};

struct Geometry {
    std::vector<uint32_t> indices;
    uint32_t opaque = 1;
    int32_t diffuse = -1, metallic_roughness = -1, normal_map = -1;
};

// Property access with the document's element named in errors.
const Json& need(const Json* v, const char* what) {
    if (!v) bad(RT_ERR_INVALID, "glTF: missing %s", what);
    return *v;
}
const Json& array_item(const Json& root, const char* key, double index) {
    const Json* a = root.get(key);
    if (!a || a->kind != Json::Arr || index < 0 || index >= (double)a->arr.size() || index != (double)(size_t)index)
        bad(RT_ERR_INVALID, "glTF: %s[%g] does not exist", key, index);
    return a->arr[(size_t)index];
}
double index_of(const Json* v, const char* what) {
    if (!v) bad(RT_ERR_INVALID, "glTF: missing %s", what);
    if (v->kind != Json::Num) bad(RT_ERR_INVALID, "glTF: %s is not an index", what);
    return v->num;
}
double num_or(const Json& o, const char* key, double dflt) {
    const Json* v = o.get(key);
    if (!v) return dflt;
    if (v->kind != Json::Num) bad(RT_ERR_INVALID, "glTF: '%s' is not a number", key);
    return v->num;
}
size_t count_of(double v, const char* what) {
    if (v < 0 || v != (double)(uint64_t)v || v > 1e15) bad(RT_ERR_INVALID, "glTF: bad %s", what);
    return (size_t)v;
}

class GltfReader {
public:
    GltfReader(const Json& doc, const uint8_t* bin, size_t bin_size) : doc_(doc), bin_(bin), bin_size_(bin_size) {}

    // Bytes of buffer view `index` (buffer 0 = the GLB binary chunk).
    std::pair<const uint8_t*, size_t> view(double index, size_t* stride) const {
        const Json& v = array_item(doc_, "bufferViews", index);
        double buffer = num_or(v, "buffer", -1);
        const Json& b = array_item(doc_, "buffers", buffer);
        if (buffer != 0 || b.get("uri") || !bin_) bad(RT_ERR_UNSUPPORTED, "glTF: buffers other than the GLB binary chunk");
        size_t off = count_of(num_or(v, "byteOffset", 0), "bufferView byteOffset");
        size_t len = count_of(num_or(v, "byteLength", -1), "bufferView byteLength");
        if (off > bin_size_ || len > bin_size_ - off) bad(RT_ERR_INVALID, "glTF: bufferView %g outside the binary chunk", index);
        if (stride) *stride = count_of(num_or(v, "byteStride", 0), "byteStride");
        return {bin_ + off, len};
    }

    struct Accessor {
        const uint8_t* base;
        size_t count, stride;
        int comps, ctype, csize;
        bool normalized;
    };

    Accessor accessor(double index) const {
        const Json& a = array_item(doc_, "accessors", index);
        if (a.get("sparse")) bad(RT_ERR_UNSUPPORTED, "glTF: sparse accessors");
        if (!a.get("bufferView")) bad(RT_ERR_UNSUPPORTED, "glTF: accessors without a bufferView");
        Accessor r;
        r.ctype = (int)num_or(a, "componentType", 0);
        switch (r.ctype) {
            case 5120: case 5121: r.csize = 1; break;
            case 5122: case 5123: r.csize = 2; break;
            case 5125: case 5126: r.csize = 4; break;
            default: bad(RT_ERR_INVALID, "glTF: accessor %g componentType %d", index, r.ctype);
        }
        const Json& t = need(a.get("type"), "accessor type");
        if (t.kind != Json::Str) bad(RT_ERR_INVALID, "glTF: accessor type");
        if (t.str == "SCALAR") r.comps = 1;
        else if (t.str == "VEC2") r.comps = 2;
        else if (t.str == "VEC3") r.comps = 3;
        else if (t.str == "VEC4") r.comps = 4;
        else bad(RT_ERR_UNSUPPORTED, "glTF: accessor type %s", t.str.c_str());
        const Json* nz = a.get("normalized");
        r.normalized = nz && nz->kind == Json::Bool && nz->b;
        r.count = count_of(num_or(a, "count", -1), "accessor count");
        size_t vstride = 0;
        auto bytes = view(num_or(a, "bufferView", -1), &vstride);
        size_t elem = (size_t)r.comps * r.csize;
        r.stride = vstride ? vstride : elem;
        if (r.stride < elem) bad(RT_ERR_INVALID, "glTF: byteStride smaller than the element");
        size_t off = count_of(num_or(a, "byteOffset", 0), "accessor byteOffset");
        if (r.count && (off > bytes.second || (r.count - 1) > (bytes.second - off) / r.stride ||
                        (r.count - 1) * r.stride + elem > bytes.second - off))
            bad(RT_ERR_INVALID, "glTF: accessor %g reads past its bufferView", index);
        r.base = bytes.first + off;
        return r;
    }

    const Json& doc_;
    const uint8_t* bin_;
    size_t bin_size_;
};

struct Model {
    std::vector<float> positions, normals, uvs;
    std::vector<Geometry> geometries;
    std::vector<Image> images;
    uint32_t primitives = 0;
};

Image single_colour(const float rgba[4]) {
    Image im;
    im.format = RT_FORMAT_R32G32B32A32_SFLOAT;
    im.filter = RT_FILTER_NEAREST;
    auto t = std::make_shared<std::vector<uint8_t>>(16);
    memcpy(t->data(), rgba, 16);
    im.texels = t;
    return im;
}

class GlbLoader {
public:
    GlbLoader(const Json& doc, const uint8_t* bin, size_t bin_size) : doc_(doc), rd_(doc, bin, bin_size) {}

    Model load() {
        Model m;
        const Json* mats = doc_.get("materials");
        size_t nmat = mats && mats->kind == Json::Arr ? mats->arr.size() : 0;
        for (size_t i = 0; i < nmat; i++) m.geometries.push_back(material(mats->arr[i], m));
        if (m.geometries.empty()) {  // util_structs.rs:1090-1111
            Geometry g;
            g.opaque = 1;
            g.diffuse = -1;   // the caller's fallback image
            const float mr[4] = {1.0f, 1.0f, 0.0f, 1.0f};
            g.metallic_roughness = push(m, single_colour(mr));
            m.geometries.push_back(std::move(g));
        }
        const Json* meshes = doc_.get("meshes");
        if (meshes && meshes->kind == Json::Arr)
            for (const Json& mesh : meshes->arr) {
                const Json* prims = mesh.get("primitives");
                if (!prims || prims->kind != Json::Arr) bad(RT_ERR_INVALID, "glTF: mesh without primitives");
                for (const Json& p : prims->arr) primitive(p, m);
            }
        return m;
    }

private:
    static int32_t push(Model& m, Image im) {
        m.images.push_back(std::move(im));
        return (int32_t)m.images.size() - 1;
    }

    // load_image_from_gltf_texture: a texture's source image decoded to RGBA8.
    Image texture(const Json& info, uint32_t format) {
        double ti = num_or(info, "index", -1);
        const Json& tex = array_item(doc_, "textures", ti);
        Image im;
        im.format = format;
        im.filter = RT_FILTER_LINEAR;
        if (const Json* s = tex.get("sampler")) {
            if (s->kind != Json::Num) bad(RT_ERR_INVALID, "glTF: texture sampler");
            const Json& smp = array_item(doc_, "samplers", s->num);
            if (num_or(smp, "magFilter", 0) == kGlNearest) im.filter = RT_FILTER_NEAREST;
        }
        double src = num_or(tex, "source", -1);
        const Json& img = array_item(doc_, "images", src);
        if (!img.get("bufferView")) bad(RT_ERR_UNSUPPORTED, "Image source is a uri which we don't support");
        size_t key = (size_t)src;
        for (const auto& c : decoded_)
            if (c.first == key) {
                im.width = c.second.width;
                im.height = c.second.height;
                im.texels = c.second.texels;
                return im;
            }
        auto bytes = rd_.view(num_or(img, "bufferView", -1), nullptr);
        auto t = std::make_shared<std::vector<uint8_t>>();
        png_decode(bytes.first, bytes.second, *t, im.width, im.height);
        im.texels = t;
        decoded_.emplace_back(key, im);
        return im;
    }

    // load_images_from_material (util_structs.rs:982-1024).
    Geometry material(const Json& mat, Model& m) {
        Geometry g;
        const Json* am = mat.get("alphaMode");
        g.opaque = !am || (am->kind == Json::Str && am->str == "OPAQUE");
        static const Json kEmpty = [] {
            Json j;
            j.kind = Json::Obj;
            return j;
        }();
        const Json* pbr = mat.get("pbrMetallicRoughness");
        if (!pbr) pbr = &kEmpty;
        if (const Json* t = pbr->get("baseColorTexture")) {
            g.diffuse = push(m, texture(*t, RT_FORMAT_R8G8B8A8_SRGB));
        } else {
            float c[4] = {1, 1, 1, 1};
            if (const Json* f = pbr->get("baseColorFactor")) {
                if (f->kind != Json::Arr || f->arr.size() != 4) bad(RT_ERR_INVALID, "glTF: baseColorFactor");
                for (int i = 0; i < 4; i++) c[i] = (float)f->arr[i].num;
            }
            g.diffuse = push(m, single_colour(c));
        }
        if (const Json* t = pbr->get("metallicRoughnessTexture")) {
            g.metallic_roughness = push(m, texture(*t, RT_FORMAT_R8G8B8A8_SRGB));
        } else {  // metallic_roughness_to_rgba (util_structs.rs:1027-1029)
            float c[4] = {1.0f, (float)num_or(*pbr, "roughnessFactor", 1.0), (float)num_or(*pbr, "metallicFactor", 1.0),
                          1.0f};
            g.metallic_roughness = push(m, single_colour(c));
        }
        if (const Json* t = mat.get("normalTexture")) g.normal_map = push(m, texture(*t, RT_FORMAT_R8G8B8A8_UNORM));
        return g;
    }

    void read_vec(const GltfReader::Accessor& a, int comps, std::vector<float>& out, const char* what) {
        if (a.comps != comps) bad(RT_ERR_INVALID, "glTF: %s must have %d components", what, comps);
        size_t at = out.size();
        out.resize(at + a.count * comps);
        float* o = out.data() + at;
        for (size_t i = 0; i < a.count; i++) {
            const uint8_t* e = a.base + i * a.stride;
            for (int c = 0; c < comps; c++) {
                float v;
                if (a.ctype == 5126) v = lef32(e + 4 * c);
                else if (a.ctype == 5121 && a.normalized) v = (float)e[c] / 255.0f;
                else if (a.ctype == 5123 && a.normalized) v = (float)le16(e + 2 * c) / 65535.0f;
                else bad(RT_ERR_UNSUPPORTED, "glTF: %s component type %d", what, a.ctype);
                o[i * comps + c] = v;
            }
        }
    }

    // One mesh primitive (util_structs.rs:1113-1137).
    void primitive(const Json& p, Model& m) {
        if (num_or(p, "mode", 4) != 4) bad(RT_ERR_UNSUPPORTED, "glTF: primitives other than triangle lists");
        double mi = num_or(p, "material", 0);
        if (mi < 0 || mi >= (double)m.geometries.size() || mi != (double)(size_t)mi)
            bad(RT_ERR_INVALID, "glTF: primitive material %g does not exist", mi);
        Geometry& g = m.geometries[(size_t)mi];
        const Json* attrs = p.get("attributes");
        if (!attrs || attrs->kind != Json::Obj) bad(RT_ERR_INVALID, "glTF: primitive without attributes");
        if (!p.get("indices")) bad(RT_ERR_UNSUPPORTED, "glTF: primitives without indices");
        auto pos = rd_.accessor(index_of(attrs->get("POSITION"), "POSITION"));
        auto nrm = rd_.accessor(index_of(attrs->get("NORMAL"), "NORMAL"));
        auto uv = rd_.accessor(index_of(attrs->get("TEXCOORD_0"), "TEXCOORD_0"));
        if (pos.ctype != 5126 || nrm.ctype != 5126) bad(RT_ERR_UNSUPPORTED, "glTF: POSITION / NORMAL must be floats");
        if (nrm.count != pos.count || uv.count != pos.count)
            bad(RT_ERR_INVALID, "glTF: POSITION, NORMAL and TEXCOORD_0 counts differ");
        size_t base = m.positions.size() / 3;
        if (base + pos.count > 0xFFFFFFFFull) bad(RT_ERR_TOO_LARGE, "glTF: more than 2^32 vertices");
        auto idx = rd_.accessor(num_or(p, "indices", -1));
        if (idx.comps != 1 || (idx.ctype != 5121 && idx.ctype != 5123 && idx.ctype != 5125))
            bad(RT_ERR_INVALID, "glTF: index accessor must be unsigned scalars");
        if (idx.count % 3) bad(RT_ERR_INVALID, "glTF: index count %zu is not a multiple of 3", idx.count);
        size_t at = g.indices.size();
        g.indices.resize(at + idx.count);
        for (size_t i = 0; i < idx.count; i++) {
            const uint8_t* e = idx.base + i * idx.stride;
            uint32_t v = idx.ctype == 5121 ? e[0] : idx.ctype == 5123 ? le16(e) : le32(e);
            if (v >= pos.count) bad(RT_ERR_INVALID, "glTF: index %u past the primitive's %zu vertices", v, pos.count);
            g.indices[at + i] = v + (uint32_t)base;
        }
        read_vec(pos, 3, m.positions, "POSITION");
        read_vec(nrm, 3, m.normals, "NORMAL");
        read_vec(uv, 2, m.uvs, "TEXCOORD_0");
        m.primitives++;
    }

    const Json& doc_;
    GltfReader rd_;
    std::vector<std::pair<size_t, Image>> decoded_;
};

Model glb_load(const uint8_t* p, size_t n) {
    if (n < 20 || le32(p) != kGlbMagic) bad(RT_ERR_INVALID, "not a GLB file");
    if (le32(p + 4) != 2) bad(RT_ERR_UNSUPPORTED, "GLB version %u", le32(p + 4));
    size_t total = le32(p + 8);
    if (total > n || total < 20) bad(RT_ERR_INVALID, "GLB length field exceeds the data");
    size_t at = 12;
    const char* json = nullptr;
    size_t json_len = 0;
    const uint8_t* bin = nullptr;
    size_t bin_len = 0;
    while (at + 8 <= total) {
        size_t len = le32(p + at);
        uint32_t type = le32(p + at + 4);
        if (len > total - at - 8) bad(RT_ERR_INVALID, "GLB chunk truncated");
        const uint8_t* d = p + at + 8;
        if (type == kChunkJson && !json) {
            json = (const char*)d;
            json_len = len;
        } else if (type == kChunkBin && !bin) {
            bin = d;
            bin_len = len;
        }
        at += 8 + ((len + 3) & ~(size_t)3);
    }
    if (!json) bad(RT_ERR_INVALID, "GLB has no JSON chunk");
    Json doc = JsonParser(json, json_len).parse();
    if (doc.kind != Json::Obj) bad(RT_ERR_INVALID, "glTF: document is not an object");
    return GlbLoader(doc, bin, bin_len).load();
}

template <class F>
int32_t guarded(F&& f) {
    try {
        return f();
    } catch (const AssetError& e) {
        return rt::report_error(e.code, "%s", e.msg.c_str());
    } catch (const std::bad_alloc&) {
        return rt::report_error(RT_ERR_OOM, "out of host memory while decoding");
    }
}

}  // namespace

struct rt_glb_model {
    Model m;
};

RTCORE_API int32_t rt_png_decode_rgba8(const void* bytes, uint64_t size, void* rgba8_out, uint64_t out_bytes,
                                       uint32_t* width, uint32_t* height) {
    return guarded([&]() -> int32_t {
        if (!bytes || !width || !height) return rt::report_error(RT_ERR_INVALID, "rt_png_decode_rgba8: null argument");
        const uint8_t* p = (const uint8_t*)bytes;
        if (!rgba8_out) {
            Png h = png_parse(p, (size_t)size, true);
            *width = h.width;
            *height = h.height;
            return RT_OK;
        }
        Png h = png_parse(p, (size_t)size, true);
        uint64_t need = (uint64_t)h.width * h.height * 4;
        if (out_bytes < need)
            return rt::report_error(RT_ERR_INVALID, "rt_png_decode_rgba8: output holds %llu bytes, %llu needed",
                                    (unsigned long long)out_bytes, (unsigned long long)need);
        std::vector<uint8_t> out;
        uint32_t w, hh;
        png_decode(p, (size_t)size, out, w, hh);
        memcpy(rgba8_out, out.data(), out.size());
        *width = w;
        *height = hh;
        return RT_OK;
    });
}

RTCORE_API int32_t rt_glb_load(const void* bytes, uint64_t size, rt_glb_model** out) {
    return guarded([&]() -> int32_t {
        if (!bytes || !out) return rt::report_error(RT_ERR_INVALID, "rt_glb_load: null argument");
        *out = nullptr;
        std::unique_ptr<rt_glb_model> m(new rt_glb_model{glb_load((const uint8_t*)bytes, (size_t)size)});
        *out = m.release();
        return RT_OK;
    });
}

RTCORE_API int32_t rt_glb_info(const rt_glb_model* model, RtGlbInfo* info) {
    if (!model || !info) return rt::report_error(RT_ERR_INVALID, "rt_glb_info: null argument");
    const Model& m = model->m;
    info->vertex_count = (uint32_t)(m.positions.size() / 3);
    info->geometry_count = (uint32_t)m.geometries.size();
    info->image_count = (uint32_t)m.images.size();
    info->primitive_count = m.primitives;
    uint64_t tris = 0;
    for (const auto& g : m.geometries) tris += g.indices.size() / 3;
    info->triangle_count = tris;
    return RT_OK;
}

RTCORE_API int32_t rt_glb_read_vertices(const rt_glb_model* model, float* positions, float* normals, float* uvs) {
    if (!model) return rt::report_error(RT_ERR_INVALID, "rt_glb_read_vertices: null model");
    const Model& m = model->m;
    if (positions) memcpy(positions, m.positions.data(), m.positions.size() * sizeof(float));
    if (normals) memcpy(normals, m.normals.data(), m.normals.size() * sizeof(float));
    if (uvs) memcpy(uvs, m.uvs.data(), m.uvs.size() * sizeof(float));
    return RT_OK;
}

RTCORE_API int32_t rt_glb_read_geometry(const rt_glb_model* model, uint32_t index, RtGlbGeometry* info,
                                        uint32_t* indices, uint64_t capacity) {
    if (!model || !info) return rt::report_error(RT_ERR_INVALID, "rt_glb_read_geometry: null argument");
    const Model& m = model->m;
    if (index >= m.geometries.size())
        return rt::report_error(RT_ERR_INVALID, "rt_glb_read_geometry: geometry %u of %zu", index, m.geometries.size());
    const Geometry& g = m.geometries[index];
    memset(info, 0, sizeof *info);
    info->index_count = (uint32_t)g.indices.size();
    info->opaque = g.opaque;
    info->diffuse_image = g.diffuse;
    info->metallic_roughness_image = g.metallic_roughness;
    info->normal_map_image = g.normal_map;
    if (indices) {
        if (capacity < g.indices.size())
            return rt::report_error(RT_ERR_INVALID, "rt_glb_read_geometry: capacity %llu < %zu indices",
                                    (unsigned long long)capacity, g.indices.size());
        memcpy(indices, g.indices.data(), g.indices.size() * sizeof(uint32_t));
    }
    return RT_OK;
}

RTCORE_API int32_t rt_glb_read_image(const rt_glb_model* model, uint32_t index, RtGlbImage* info, void* texels,
                                     uint64_t capacity) {
    if (!model || !info) return rt::report_error(RT_ERR_INVALID, "rt_glb_read_image: null argument");
    const Model& m = model->m;
    if (index >= m.images.size())
        return rt::report_error(RT_ERR_INVALID, "rt_glb_read_image: image %u of %zu", index, m.images.size());
    const Image& im = m.images[index];
    info->width = im.width;
    info->height = im.height;
    info->format = im.format;
    info->filter = im.filter;
    info->byte_size = im.texels->size();
    if (texels) {
        if (capacity < im.texels->size())
            return rt::report_error(RT_ERR_INVALID, "rt_glb_read_image: capacity %llu < %zu bytes",
                                    (unsigned long long)capacity, im.texels->size());
        memcpy(texels, im.texels->data(), im.texels->size());
    }
    return RT_OK;
}

RTCORE_API int32_t rt_glb_destroy(rt_glb_model* model) {
    delete model;
    return RT_OK;
}
