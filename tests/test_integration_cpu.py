"""The Rust binding written out in INTEGRATION.md (the `cellsim-sys` crate a maintainer would add
to the reference; it cannot be compiled here) against include/cellsim.h: every function and every
struct of the header appears in the `extern "C"` block and the `#[repr(C)]` structs, with the same
parameters, field order and the C types mapped to their Rust FFI equivalents.  This keeps the
unbuilt binding from drifting away from the ABI."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "cellsim.h"
INTEGRATION = ROOT / "INTEGRATION.md"

BASE = {"uint8_t": "u8", "uint32_t": "u32", "int32_t": "i32", "uint64_t": "u64", "int64_t": "i64", "float": "f32",
        "char": "c_char", "void": "c_void", "cs_status": "cs_status"}


def _clean_header():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return re.sub(r"//[^\n]*", "", text)


def c_to_rust(ctype: str) -> str:
    """FFI spelling of a C parameter or field type: T* -> *mut T, const T* -> *const T."""
    t = " ".join(ctype.replace("*", " * ").split())
    toks = t.split(" ")
    base_const = toks[0] == "const"
    if base_const:
        toks = toks[1:]
    base = toks[0]
    rust = BASE.get(base, base)
    ptr_quals = []  # per '*', whether the pointer it forms points to const
    pending_const = base_const
    for tok in toks[1:]:
        if tok == "*":
            ptr_quals.append(pending_const)
            pending_const = False
        elif tok == "const":
            pending_const = True
    for is_const in ptr_quals:
        rust = f"*{'const' if is_const else 'mut'} {rust}"
    return rust


def parse_header_functions():
    """[(name, return type, [(param type, param name)])] of every cs_ function."""
    text = _clean_header()
    out = []
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(cs_[a-z_0-9]+)\s*\(([^)]*)\)\s*;", text):
        ret = " ".join(m.group(1).split())
        params = []
        args = m.group(3).strip()
        if args and args != "void":
            for a in args.split(","):
                a = " ".join(a.replace("*", " * ").split())
                pm = re.match(r"(.*?)\s*([A-Za-z_]\w*)$", a)
                params.append((pm.group(1).strip(), pm.group(2)))
        out.append((m.group(2), ret, params))
    return out


def parse_header_structs():
    """{name: [(field, type, array length or None)]} of every typedef struct."""
    text = _clean_header()
    out = {}
    for m in re.finditer(r"typedef\s+struct\s*\{(.*?)\}\s*(\w+)\s*;", text, flags=re.S):
        fields = []
        for decl in m.group(1).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            dm = re.match(r"((?:const\s+)?[A-Za-z_]\w*(?:\s*\*)*)\s*(.*)$", decl)
            base, rest = dm.group(1), dm.group(2)
            for item in rest.split(","):
                item = item.strip()
                stars = item.count("*")
                item = item.replace("*", "").strip()
                am = re.match(r"(\w+)(?:\[(\d+)\])?$", item)
                fields.append((am.group(1), base + " *" * stars, am.group(2)))
        out[m.group(2)] = fields
    return out


def _rust_blocks():
    text = INTEGRATION.read_text()
    blocks = re.findall(r"```rust\n(.*?)```", text, flags=re.S)
    return "\n".join(blocks)


def parse_rust_functions():
    rust = _rust_blocks()
    ext = re.search(r'extern "C" \{(.*?)\n\}', rust, flags=re.S).group(1)
    out = {}
    for m in re.finditer(r"pub fn (\w+)\((.*?)\)\s*(?:->\s*([^;]+))?;", ext, flags=re.S):
        params = []
        for a in [x.strip() for x in m.group(2).split(",") if x.strip()]:
            n, t = a.split(":", 1)
            params.append((n.strip(), " ".join(t.split())))
        out[m.group(1)] = (params, (m.group(3) or "").strip() or "void")
    return out


def parse_rust_structs():
    rust = _rust_blocks()
    out = {}
    for m in re.finditer(r"#\[repr\(C\)\]\s*pub struct (\w+)\s*\{(.*?)\}", rust, flags=re.S):
        fields = []
        for f in [x.strip() for x in m.group(2).replace("\n", " ").split(",") if x.strip()]:
            n, t = f.replace("pub ", "", 1).split(":", 1)
            fields.append((n.strip(), " ".join(t.split())))
        out[m.group(1)] = fields
    return out


def test_rust_extern_block_matches_header():
    header = parse_header_functions()
    rust = parse_rust_functions()
    assert len(header) >= 50
    missing = [n for n, _, _ in header if n not in rust]
    assert not missing, f"functions of cellsim.h missing from the Rust binding: {missing}"
    extra = sorted(set(rust) - {n for n, _, _ in header})
    assert not extra, f"Rust binding declares functions cellsim.h does not: {extra}"
    for name, ret, params in header:
        rparams, rret = rust[name]
        assert len(rparams) == len(params), (name, params, rparams)
        for (ctype, cname), (rname, rtype) in zip(params, rparams):
            assert rtype == c_to_rust(ctype), (name, cname, ctype, rtype)
        want_ret = "void" if ret == "void" else c_to_rust(ret)
        assert rret == want_ret, (name, ret, rret)


def test_rust_structs_match_header():
    header = parse_header_structs()
    rust = parse_rust_structs()
    for name in ("cs_lattice_params", "cs_region_desc", "cs_info", "cs_stat_sample", "cs_ref_frame_noalloc_args"):
        assert name in header and name in rust, name
        hf, rf = header[name], rust[name]
        assert [("type_" if f == "type" else f) for f, _, _ in hf] == [n for n, _ in rf], name
        for (f, ctype, arr), (_, rtype) in zip(hf, rf):
            want = c_to_rust(ctype)
            if arr:
                want = f"[{want}; {arr}]"
            assert rtype == want, (name, f, ctype, rtype)


def test_type_mapping():
    assert c_to_rust("const char* const*") == "*const *const c_char"
    assert c_to_rust("cs_sim**") == "*mut *mut cs_sim"
    assert c_to_rust("const cs_sim*") == "*const cs_sim"
    assert c_to_rust("uint32_t") == "u32"
    assert c_to_rust("void*") == "*mut c_void"
