"""The Rust binding a maintainer would add to the reference's host
(ray-tracing-gallery_gb300/rtcore-sys, source only: no Rust toolchain here)
declares every function the C headers export, with the same number of
parameters, and restates the headers' struct sizes."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
LIB_RS = ROOT / "ray-tracing-gallery_gb300" / "rtcore-sys" / "src" / "lib.rs"


def _c_functions():
    out = {}
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"RTCORE_API\s+[\w\s\*]+?\b(rt_\w+)\s*\(([^)]*)\)\s*;", text):
            args = [a for a in m.group(2).split(",") if a.strip() and a.strip() != "void"]
            out[m.group(1)] = len(args)
    return out


def _rust_functions():
    text = LIB_RS.read_text()
    out = {}
    for m in re.finditer(r"pub fn (rt_\w+)\s*\(([^)]*)\)", text, flags=re.S):
        args = [a for a in m.group(2).split(",") if a.strip()]
        out[m.group(1)] = len(args)
    return out


def test_every_exported_function_is_bound_with_its_arity():
    c, rust = _c_functions(), _rust_functions()
    assert len(c) >= 39
    missing = sorted(set(c) - set(rust))
    assert not missing, f"not bound in rtcore-sys: {missing}"
    wrong = {k: (c[k], rust[k]) for k in c if rust[k] != c[k]}
    assert not wrong, f"parameter counts differ (C, Rust): {wrong}"


def test_struct_sizes_match_the_header_asserts():
    header = (ROOT / "include" / "rtcore.h").read_text()
    sizes = dict(re.findall(r"sizeof\((Rt\w+)\) == (\d+)", header))
    rust = dict(re.findall(r"size_of::<(Rt\w+)>\(\) == (\d+)", LIB_RS.read_text()))
    shared = set(sizes) & set(rust)
    assert len(shared) >= 12
    assert all(sizes[k] == rust[k] for k in shared), {k: (sizes[k], rust[k]) for k in shared}
