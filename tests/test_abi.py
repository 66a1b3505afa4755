"""CPU tests of the C ABI: layouts, exported symbols, host-side validation.
No compute call is made here (there is no GPU on this side)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from rtgallery import abi

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions() -> set[str]:
    names = set()
    for h in HEADERS:
        names |= set(re.findall(r"RTCORE_API\s+[\w\s\*]+?\b(rt_\w+)\s*\(", h.read_text()))
    return names


def test_layouts_match_reference():
    abi.check_layouts()


def test_header_constants_match_the_python_binding():
    """Every integer #define RT_* of the headers (a literal or `(a << b)`)
    exists in the ctypes binding with the same value."""
    seen = 0
    for h in HEADERS:
        for m in re.finditer(r"^#define\s+(RT_[A-Z0-9_]+)\s+(.+?)\s*(?:/\*.*)?$", h.read_text(), re.M):
            name, body = m.group(1), m.group(2)
            lit = re.fullmatch(r"\(?(0x[0-9a-fA-F]+|\d+)u?l{0,2}\)?", body)
            shl = re.fullmatch(r"\((\d+)u?l{0,2}\s*<<\s*(\d+)\)", body)
            if not (lit or shl):
                continue
            value = int(lit.group(1), 0) if lit else int(shl.group(1)) << int(shl.group(2))
            assert hasattr(abi, name), f"{h.name}: {name} missing from abi.py"
            assert getattr(abi, name) == value, (h.name, name, getattr(abi, name), value)
            seen += 1
    assert seen >= 60


def test_header_static_asserts_compile(tmp_path):
    src = tmp_path / "t.c"
    src.write_text("".join(f'#include "{h.name}"\n' for h in HEADERS) + "int main(void){return 0;}\n")
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src), "-o",
                        str(tmp_path / "t")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(["g++", "-std=c++17", "-Wall", "-Werror", "-x", "c++", "-I", str(ROOT / "include"), str(src),
                        "-o", str(tmp_path / "t2")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_library_exports_every_declared_symbol(rtlib):
    declared = declared_functions()
    assert len(declared) >= 17
    assert declared == set(abi.EXPORTED_FUNCTIONS), declared ^ set(abi.EXPORTED_FUNCTIONS)
    out = subprocess.run(["nm", "-D", "--defined-only", str(abi.library_path())], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert declared <= exported
    # only the ABI is exported from our code (cudart's own symbols aside)
    ours = {s for s in exported if s.startswith("rt_")}
    assert ours == declared
    for name in declared:
        assert hasattr(rtlib, name)


def test_version_string(rtlib):
    assert b"sm_103a" in rtlib.rt_version_string()


def test_blas_size_query_validates_on_host(rtlib):
    g = (abi.RtGeometryTriangles * 2)()
    g[0].vertex_address = 4096
    g[0].index_address = 8192
    g[0].vertex_stride = 12
    g[0].max_vertex = 99
    g[0].primitive_count = 1000
    g[1].vertex_address = 4096
    g[1].vertex_stride = 12
    g[1].primitive_count = 24
    s = abi.RtBuildSizes()
    assert rtlib.rt_get_blas_build_sizes(g, 2, 0, C.byref(s)) == abi.RT_OK
    assert s.acceleration_structure_size >= 512 + 1024 * 48 and s.acceleration_structure_size % 256 == 0
    assert s.build_scratch_size > 0
    g[0].vertex_stride = 10
    assert rtlib.rt_get_blas_build_sizes(g, 2, 0, C.byref(s)) == abi.RT_ERR_INVALID
    assert b"vertex_stride" in rtlib.rt_last_error_string()
    assert rtlib.rt_get_blas_build_sizes(g, 129, 0, C.byref(s)) == abi.RT_ERR_TOO_LARGE
    g[0].vertex_stride = 12
    g[0].primitive_count = 1 << 28
    assert rtlib.rt_get_blas_build_sizes(g, 2, 0, C.byref(s)) == abi.RT_ERR_TOO_LARGE


def test_tlas_size_query(rtlib):
    a, b = abi.RtBuildSizes(), abi.RtBuildSizes()
    assert rtlib.rt_get_tlas_build_sizes(256, 0, C.byref(a)) == 0
    assert rtlib.rt_get_tlas_build_sizes(4096, 0, C.byref(b)) == 0
    assert b.acceleration_structure_size > a.acceleration_structure_size
    assert a.update_scratch_size < a.build_scratch_size
    assert rtlib.rt_get_tlas_build_sizes(0, 0, C.byref(a)) == 0


def test_null_and_alignment_rejected_before_launch(rtlib):
    assert rtlib.rt_ctx_create(0, None) == abi.RT_ERR_INVALID
    s = abi.RtBuildSizes()
    assert rtlib.rt_get_tlas_build_sizes(4, 0, None) == abi.RT_ERR_INVALID
    # misaligned destination: rejected on the host, nothing is launched
    assert rtlib.rt_cmd_build_tlas(None, 16, 4, 0, 4096 + 16, 1 << 20, 8192, 1 << 20, None) == abi.RT_ERR_INVALID
    assert rtlib.rt_cmd_copy_acceleration_structure(None, 256, 256, 4096, 0, None) == abi.RT_ERR_INVALID
    assert rtlib.rt_get_acceleration_structure_device_address(4096 + 8) == 0
    assert rtlib.rt_get_acceleration_structure_device_address(4096) == 4096
    assert rtlib.rt_debug_eval(99, 0, 0, 0, None) == abi.RT_ERR_INVALID
    del s


def _static_scratch_limit(rtlib, flags: int) -> int:
    """Largest triangle count whose BLAS build scratch fits the library's
    static scratch array (rt_cmd_build_blas_static_scratch), by the size query."""
    def fits(n):
        g = (abi.RtGeometryTriangles * 1)()
        g[0].vertex_address = 4096
        g[0].index_address = 8192
        g[0].vertex_stride = 12
        g[0].max_vertex = 3 * n
        g[0].primitive_count = n
        s = abi.RtBuildSizes()
        assert rtlib.rt_get_blas_build_sizes(g, 1, flags, C.byref(s)) == abi.RT_OK
        return s.build_scratch_size <= abi.RT_STATIC_SCRATCH_BYTES

    lo, hi = 1, 4 << 20
    while lo < hi:
        mid = (lo + hi + 1) // 2
        lo, hi = (mid, hi) if fits(mid) else (lo, mid - 1)
    return lo


def test_static_scratch_limits_match_the_documentation(rtlib):
    """The triangle limits the header states for the allocation-free build
    (about 288k with PREFER_FAST_TRACE, about 462k without) follow from the
    size query, within 1 %."""
    text = (ROOT / "include" / "rtcore.h").read_text()
    assert "about 288k triangles" in text and "about 462k otherwise" in text
    fast_trace = _static_scratch_limit(rtlib, abi.RT_BUILD_PREFER_FAST_TRACE)
    plain = _static_scratch_limit(rtlib, 0)
    assert abs(fast_trace - 288_000) <= 2_880, fast_trace
    assert abs(plain - 462_000) <= 4_620, plain
