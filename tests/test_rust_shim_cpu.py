"""The Rust binding (bwa-cuda/, a crate for the bwa-mem4 workspace) against the C ABI.

No Rust toolchain exists on these machines, so the crate is not compiled; these checks read its
source instead: every extern "C" declaration of bwa-cuda/src/lib.rs names a symbol that
libbwacuda.so exports and that include/bwacuda.h declares, with the header's argument count, and
every #[repr(C)] struct of the binding lists the header struct's fields in the header's order."""
import ctypes
import os
import re

import pytest

import bwacuda as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.usefixtures("built")


def _strip_c_comments(src):
    return re.sub(r"/\*.*?\*/", "", src, flags=re.S)


def _nargs(arglist):
    a = arglist.strip()
    if a in ("", "void"):
        return 0
    return a.count(",") + 1


def _header_functions():
    src = _strip_c_comments(open(os.path.join(ROOT, "include", "bwacuda.h")).read())
    out = {}
    for name, args in re.findall(r"\b(bwacuda_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src):
        out[name] = _nargs(args)
    return out


def _rust_source():
    return open(os.path.join(ROOT, "bwa-cuda", "src", "lib.rs")).read()


def _rust_functions():
    src = _rust_source()
    blocks = re.findall(r'extern "C" \{(.*?)\n    \}', src, flags=re.S)
    assert blocks, "no extern block in bwa-cuda/src/lib.rs"
    out = {}
    for blk in blocks:
        for name, args in re.findall(r"pub fn (bwacuda_[a-z0-9_]+)\((.*?)\)", blk, flags=re.S):
            out[name] = _nargs(args)
    return out


def _header_structs():
    src = _strip_c_comments(open(os.path.join(ROOT, "include", "bwacuda.h")).read())
    out = {}
    for body, name in re.findall(r"typedef struct \{(.*?)\}\s*(bwacuda_[a-z0-9_]+)\s*;", src, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            # "type a, b, c" / "const uint8_t *query" / "int8_t mat[64]" / "bwacuda_rescue_result aln"
            first, *rest = decl.split(",")
            names = [re.findall(r"([A-Za-z_][A-Za-z0-9_]*)\s*(?:\[\d+\])?\s*$", first)[0]]
            names += [r.strip().lstrip("*").split("[")[0].strip() for r in rest]
            fields += names
        out[name] = fields
    return out


def _rust_structs():
    src = _rust_source()
    out = {}
    for name, body in re.findall(r"pub struct (bwacuda_[a-z0-9_]+) \{(.*?)\}", src, flags=re.S):
        out[name] = re.findall(r"pub ([a-z0-9_]+):", body)
    return out


def test_crate_files_present():
    for rel in ("Cargo.toml", "build.rs", os.path.join("src", "lib.rs")):
        assert os.path.isfile(os.path.join(ROOT, "bwa-cuda", rel)), rel
    toml = open(os.path.join(ROOT, "bwa-cuda", "Cargo.toml")).read()
    assert 'links = "bwacuda"' in toml and "bwa-extend" in toml and "bwa-neon" in toml
    assert "rustc-link-lib=dylib=bwacuda" in open(os.path.join(ROOT, "bwa-cuda", "build.rs")).read()


def test_every_declaration_is_exported_with_the_header_arity():
    lib = ctypes.CDLL(B.LIB_PATH)
    hdr = _header_functions()
    rs = _rust_functions()
    assert rs, "no declarations parsed"
    for name, n in rs.items():
        assert hasattr(lib, name), f"{name} is not exported by libbwacuda.so"
        assert name in hdr, f"{name} is not declared in include/bwacuda.h"
        assert n == hdr[name], f"{name}: {n} arguments in the binding, {hdr[name]} in the header"
    # the binding covers the whole ABI
    assert set(rs) == set(hdr)


def test_structs_match_the_header_field_for_field():
    hdr = _header_structs()
    rs = _rust_structs()
    assert "bwacuda_ext_job" in rs and "bwacuda_rescue_result" in rs
    opaque = {"bwacuda_ctx"}  # declared in the header as an incomplete type
    for name, fields in rs.items():
        if name in opaque:
            continue
        assert name in hdr, f"{name} is not a header struct"
        assert fields == hdr[name], f"{name}: {fields} vs {hdr[name]}"
    assert set(hdr) <= set(rs), f"header structs missing from the binding: {set(hdr) - set(rs)}"


def test_reference_facing_items():
    src = _rust_source()
    # the trait the reference's run_side is generic over, and the free function pe.rs calls
    assert re.search(r"impl SwBackend for CudaBackend", src)
    for fn in ("fn name(&self)", "fn extend(", "fn extend_batch(", "pub fn batched_ksw_align2(",
               "pub fn ksw_align2("):
        assert fn in src, fn
    sig = re.search(r"pub fn batched_ksw_align2\((.*?)\) -> Vec<KswAlignResult>", src, flags=re.S).group(1)
    names = re.findall(r"([a-z_0-9]+):", sig)
    # crates/bwa-neon/src/matesw.rs:299-309
    assert names == ["jobs", "m", "mat", "o_del", "e_del", "o_ins", "e_ins", "minsc", "max_sc"]
