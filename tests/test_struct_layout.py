"""The ctypes mirrors of the C ABI's structs (meshlesshydro_gb300/runtime.py,
config.py) declare the same fields, in the same order, with the same types as
include/mlh.h: a field added on one side only would shift every later field
without any error at the call."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

C_TYPES = {"int": ctypes.c_int, "unsigned int": ctypes.c_uint, "double": ctypes.c_double,
           "long long": ctypes.c_longlong}


def header_structs():
    """{struct name: [(field, ctypes type), ...]} of the typedef'd structs."""
    src = open(os.path.join(ROOT, "include", "mlh.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for name, body in re.findall(r"typedef struct (\w+) \{(.*?)\} \1;", src, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"(const )?(unsigned int|long long|int|double)\s*(.*)", decl)
            assert m, (name, decl)
            base = C_TYPES[m.group(2)]
            for part in m.group(3).split(","):
                part = part.strip()
                ptr = part.startswith("*")
                part = part.lstrip("*").strip()
                arr = re.match(r"(\w+)\[(\d+)\]", part)
                if arr:
                    fields.append((arr.group(1), base * int(arr.group(2))))
                else:
                    fields.append((part, ctypes.POINTER(base) if ptr else base))
        out[name] = fields
    return out


def _same(a, b):
    if a is b:
        return True
    if hasattr(a, "_length_") and hasattr(b, "_length_"):
        return a._length_ == b._length_ and a._type_ is b._type_
    if hasattr(a, "_type_") and hasattr(b, "_type_") and a.__name__.startswith("LP_"):
        return b.__name__.startswith("LP_") and a._type_ is b._type_
    return False


@pytest.mark.parametrize("cname,pyname", [("mlh_config", "config.CConfig"),
                                          ("mlh_particles_view", "runtime.ParticlesView"),
                                          ("mlh_step_stats", "runtime.StepStats"),
                                          ("mlh_member", "runtime.MemberDesc"),
                                          ("mlh_tuning", "runtime.Tuning")])
def test_ctypes_mirrors_match_header(cname, pyname):
    import importlib
    mod, cls = pyname.split(".")
    py = getattr(importlib.import_module("meshlesshydro_gb300." + mod), cls)
    want = header_structs()[cname]
    got = list(py._fields_)
    assert [f for f, _ in got] == [f for f, _ in want], cname
    for (f, a), (_, b) in zip(got, want):
        assert _same(a, b), (cname, f, a, b)
