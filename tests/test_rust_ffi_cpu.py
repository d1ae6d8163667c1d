"""The Rust FFI crate (crates/gvs-sys) against the C ABI (include/gvs.h), without a Rust
toolchain: every function the header declares is declared in the crate's extern block
with the same argument names, count and types (C -> Rust mapping below), the three
structs have the same fields in the same order with the same types, and build.rs
compiles with the same nvcc flags as the Python build (gravis_gb300/build.py).
"""
import os
import re

from gravis_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "gvs.h")
SYS = os.path.join(ROOT, "crates", "gvs-sys", "src", "lib.rs")
BUILD_RS = os.path.join(ROOT, "crates", "gvs-sys", "build.rs")
SAFE = os.path.join(ROOT, "crates", "gvs", "src", "lib.rs")

C2R = {"size_t": "usize", "int": "c_int", "double": "f64", "float": "f32", "unsigned": "c_uint",
       "long long": "c_longlong", "uint8_t": "u8", "uint32_t": "u32", "uint64_t": "u64", "int64_t": "i64",
       "char": "c_char", "void": "c_void", "gvs_status": "gvs_status", "gvs_ctx": "gvs_ctx", "gvs_diag": "gvs_diag",
       "gvs_sph_params": "gvs_sph_params", "gvs_profile": "gvs_profile"}


def rust_type(ctype: str) -> str:
    ctype = " ".join(ctype.split())
    const = ctype.startswith("const ")
    if const:
        ctype = ctype[6:]
    stars = ctype.count("*")
    r = C2R[ctype.replace("*", "").strip()]
    for k in range(stars):
        r = ("*const " if const and k == 0 else "*mut ") + r
    return r


def header_functions():
    body = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for ret, name, args in re.findall(r"((?:const\s+)?[a-z_0-9]+\s*\*?\s*)\b(gvs_[a-z0-9_]+)\s*\(([^;{]*?)\)\s*;",
                                      body, flags=re.S):
        params = []
        args = " ".join(args.split())
        if args and args != "void":
            for a in args.split(","):
                m = re.match(r"(.*?)([A-Za-z_][A-Za-z_0-9]*)$", a.strip())
                pname = "ptype" if m.group(2) == "type" else m.group(2)
                params.append((pname, rust_type(m.group(1))))
        out[name] = (params, rust_type(ret))
    return out


def rust_functions():
    src = open(SYS).read()
    block = src[src.index('unsafe extern "C" {'):]
    block = block[: block.index("\n}\n")]
    out = {}
    for name, args, ret in re.findall(r"pub fn (gvs_[a-z0-9_]+)\((.*?)\)\s*->\s*([^;]+);", block, flags=re.S):
        params = []
        args = " ".join(args.split())
        if args:
            for a in args.split(","):
                a = a.strip()
                if a:
                    pn, ty = a.split(":", 1)
                    params.append((pn.strip(), " ".join(ty.split())))
        out[name] = (params, " ".join(ret.split()))
    return out


def test_every_header_function_is_declared_in_the_sys_crate():
    h, r = header_functions(), rust_functions()
    assert len(h) >= 50
    assert sorted(h) == sorted(r), (sorted(set(h) ^ set(r)))
    for name, (params, ret) in h.items():
        rp, rret = r[name]
        assert rret == ret, (name, rret, ret)
        assert rp == params, (name, rp, params)


def struct_fields_c(name):
    body = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    m = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), body, flags=re.S)
    fields = []
    for decl in m.group(1).split(";"):
        decl = " ".join(decl.split())
        if not decl:
            continue
        parts = decl.split(" ")
        if parts[0] == "long" and parts[1] == "long":
            ctype, names = "long long", " ".join(parts[2:])
        else:
            ctype, names = parts[0], " ".join(parts[1:])
        for nm in names.split(","):
            nm = nm.strip()
            arr = re.match(r"(\w+)\[(\d+)\]", nm)
            if arr:
                fields.append((arr.group(1), f"[{C2R[ctype]}; {arr.group(2)}]"))
            else:
                fields.append((nm, C2R[ctype]))
    return fields


def struct_fields_rust(name):
    src = open(SYS).read()
    m = re.search(r"pub struct %s \{(.*?)\n\}" % name, src, flags=re.S)
    return [(a.strip(), " ".join(b.split())) for a, b in re.findall(r"pub (\w+):\s*([^,\n]+),", m.group(1))]


def test_struct_layouts_match():
    for name in ("gvs_diag", "gvs_sph_params", "gvs_profile"):
        assert struct_fields_rust(name) == struct_fields_c(name), name


def test_status_and_enum_constants_match():
    h = open(HEADER).read()
    src = open(SYS).read()
    for cname, value in re.findall(r"\b(GVS_[A-Z0-9_]+)\s*=\s*(\d+)", h):
        m = re.search(r"pub const %s: \w+ = (\d+);" % cname, src)
        assert m and m.group(1) == value, cname


def test_build_rs_uses_the_python_build_flags():
    src = open(BUILD_RS).read()

    def rs_list(const):
        m = re.search(r"const %s: &\[&str\] = &\[(.*?)\];" % const, src, flags=re.S)
        return re.findall(r'"([^"]*)"', m.group(1))

    assert rs_list("ARCH") == B.ARCH
    assert rs_list("NVCC_FLAGS") == B.NVCC_FLAGS
    file_flags = dict((f, re.findall(r'"([^"]*)"', fl)) for f, fl in
                      re.findall(r'\("([^"]+)", &\[(.*?)\]\)', src[src.index("const FILE_FLAGS"):]))
    assert file_flags == B.FILE_FLAGS
    assert "arch=compute_103a,code=sm_103a" in src and "cudart_static" in src


def test_safe_crate_implements_the_sim_core_traits():
    src = open(SAFE).read()
    assert "impl GravitySolver for GpuGravity" in src
    assert "impl Integrator for GpuLeapfrog" in src
    for fn in ("pub fn compute(", "pub fn compute_timestep(", "pub fn step_with_sph(", "pub fn gravity_for("):
        assert fn in src, fn
    called = set(re.findall(r"sys::(gvs_[a-z0-9_]+)\(", src))
    assert called <= set(header_functions()), called - set(header_functions())
