"""The Fortran modules (magic_gb300/fortran/*.f90) bind the C ABI through
ISO_C_BINDING; no Fortran compiler exists here, so these tests check the
bindings as text: every bind(C) name is an entry point include/magic_sht.h
declares, and every bind(C) derived type has the components of the C struct
of the same name in the same order with matching kinds."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "magic_sht.h")
F90 = sorted(glob.glob(os.path.join(ROOT, "magic_gb300", "fortran", "*.f90")))


def c_structs():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for name, body in re.findall(r"typedef struct (\w+)\s*\{(.*?)\}\s*\1\s*;", src, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = decl.strip()
            if not decl:
                continue
            m = re.match(r"((?:const\s+)?(?:long long|double|int|void))\s+(.*)", decl)
            assert m, decl
            base = m.group(1).replace("const ", "")
            for v in m.group(2).split(","):
                v = v.strip()
                kind = "ptr" if v.startswith("*") else {"long long": "i64", "double": "f64", "int": "i32"}[base]
                # arrays: name[4] in C, name(4) in Fortran
                fields.append((v.lstrip("*").strip().lower().replace("[", "(").replace("]", ")"), kind))
        out[name] = fields
    return out


def f_types():
    out = {}
    kinds = {"type(c_ptr)": "ptr", "integer(c_long_long)": "i64", "real(c_double)": "f64", "integer(c_int)": "i32"}
    for path in F90:
        src = open(path).read()
        for name, body in re.findall(r"type, bind\(C\) :: (\w+)\n(.*?)end type", src, flags=re.S | re.I):
            fields = []
            for line in body.splitlines():
                line = line.split("!")[0].strip()
                if not line:
                    continue
                decl, names = line.split("::")
                kind = kinds[decl.strip().lower()]
                fields += [(n.strip().lower(), kind) for n in names.split(",")]
            out.setdefault(name, []).append((path, fields))
    return out


def test_bind_names_are_declared():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    declared = set(re.findall(r"\b(magic_sht_\w+)\s*\(", src))
    names = set()
    for path in F90:
        names |= set(re.findall(r"bind\(C,\s*name='(\w+)'\)", open(path).read()))
    assert names, "no bindings found"
    assert names <= declared, sorted(names - declared)
    # the batched radial-loop entry points are bound
    for n in ("magic_sht_transform_to_grid_space", "magic_sht_transform_to_lm_space", "magic_sht_get_nl",
              "magic_sht_get_td_nbc", "magic_sht_courant", "magic_sht_dt_courant"):
        assert n in names, n


def test_bind_types_match_c_structs():
    cs = c_structs()
    ft = f_types()
    assert ft, "no bind(C) types found"
    for name, defs in ft.items():
        assert name in cs, name
        for path, fields in defs:
            assert fields == cs[name], (os.path.basename(path), name, fields, cs[name])


def test_precision_switch_matches_header():
    """MAGIC_SHT_PRECISION in the drop-in's initialize_sht maps each form name
    to the MAGIC_SHT_* value of the header, and the Python names agree."""
    from magic_gb300 import _lib
    hdr = open(HEADER).read()
    consts = {m.group(1).lower(): int(m.group(2))
              for m in re.finditer(r"#define MAGIC_SHT_(FP64|FP32|BF16X3|TF32X2|FP64TC|BF16X5)\s+(\d+)", hdr)}
    src = open(os.path.join(ROOT, "magic_gb300", "fortran", "sht_gpu.f90")).read()
    cases = {m.group(1): int(m.group(2))
             for m in re.finditer(r"case \( '(\w+)' \)\s*\n\s*d%precision = (\d+)", src)}
    assert cases == consts, (cases, consts)
    assert {k: _lib.PRECISIONS[k] for k in consts} == consts
