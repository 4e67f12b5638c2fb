"""The C-ABI library loads and exports every symbol include/*.h declares;
the ctypes mirror and the Fortran interface module repeat the C structures
member for member (names, order, kinds, offsets as compiled)."""
import ctypes as C
import os
import re

from sem2dpack_gb300 import _lib, abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_functions():
    names = set()
    for h in ("sem2d_gpu.h", "sem2d_host.h"):
        src = open(os.path.join(INCLUDE, h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(sem2d_\w+)\s*\(", src):
            names.add(m.group(1))
    return names


def c_structs(header):
    """{struct name: [(member, base type, pointer depth, array length)]}
    of the typedef'd structures of a header, in declaration order."""
    src = open(os.path.join(INCLUDE, header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for m in re.finditer(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", src, flags=re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            mm = re.match(r"((?:const\s+)?(?:unsigned\s+)?\w+)\s+(.*)", decl)
            base = mm.group(1).replace("const ", "")
            for d in mm.group(2).split(","):
                ptr = d.count("*")
                d = d.replace("*", "").strip()
                am = re.match(r"(\w+)\s*\[(\w+)\]", d)
                arr = None
                if am:
                    d, arr = am.group(1), am.group(2)
                fields.append((d, base, ptr, arr))
        out[m.group(3)] = fields
    return out


def fortran_types():
    """{type name: [(member, fortran type, dims)]} of the bind(C) types of
    include/sem2d_gpu_iface.f90."""
    src = open(os.path.join(INCLUDE, "sem2d_gpu_iface.f90")).read()
    out = {}
    for m in re.finditer(r"type, bind\(C\) :: (\w+)\n(.*?)\n\s*end type", src, flags=re.S):
        fields = []
        for line in m.group(2).split("\n"):
            t, _, decl = line.partition("::")
            dm = re.match(r"\s*(\w+)\s*(?:\((\w+)\))?", decl)
            fields.append((dm.group(1), " ".join(t.split()), dm.group(2)))
        out[m.group(1)] = fields
    return out


def test_all_declared_symbols_exported():
    L = _lib.lib()
    names = declared_functions()
    assert len(names) > 25
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    # and the ctypes prototype table covers exactly the declared functions
    assert {p[0] for p in _lib.PROTOTYPES} == names


def test_struct_layouts_match():
    a, b = C.c_int(), C.c_int()
    assert _lib.lib().sem2d_abi_struct_sizes(C.byref(a), C.byref(b)) == 0
    assert a.value == C.sizeof(abi.ProblemDesc)
    assert b.value == C.sizeof(abi.Deck)


def _offsets(which):
    L = _lib.lib()
    n = L.sem2d_abi_field_offsets(which, None, 0)
    assert n > 0
    out = (C.c_longlong * n)()
    assert L.sem2d_abi_field_offsets(which, out, n) == n
    return list(out)


def test_every_member_offset_matches():
    """Names and order of the ctypes mirror against the header, offsets
    against the compiled library: two members swapped with equal sizes
    fail here."""
    structs = {**c_structs("sem2d_gpu.h"), **c_structs("sem2d_host.h")}
    for which, (cname, py) in enumerate([("sem2d_problem_desc", abi.ProblemDesc), ("sem2d_deck", abi.Deck),
                                         ("sem2d_lattice_args", abi.LatticeArgs), ("sem2d_stf", abi.Stf)]):
        header = [f[0] for f in structs[cname]]
        mirror = [f[0] for f in py._fields_]
        assert header == mirror, cname
        offs = _offsets(which)
        assert len(offs) == len(header), cname
        for name, off in zip(header, offs):
            assert getattr(py, name).offset == off, (cname, name)
    assert _lib.lib().sem2d_abi_field_offsets(7, None, 0) == abi.SEM2D_E_ARG


def test_fortran_types_repeat_the_header():
    structs = c_structs("sem2d_gpu.h")
    ftypes = fortran_types()
    kinds = {"int": "integer(c_int)", "double": "real(c_double)", "char": "character(kind=c_char)"}
    for name in ("sem2d_stf", "sem2d_problem_desc", "sem2d_lattice_args"):
        c, f = structs[name], ftypes[name]
        assert [m[0] for m in c] == [m[0] for m in f], name
        for (cn, base, ptr, arr), (fn, ft, fdim) in zip(c, f):
            assert ft == ("type(c_ptr)" if ptr else kinds[base]), (name, cn)
            assert fdim == arr, (name, cn)


def test_fortran_interfaces_cover_the_header():
    src = open(os.path.join(INCLUDE, "sem2d_gpu_iface.f90")).read()
    bound = set(re.findall(r'bind\(C, name="(sem2d_\w+)"\)', src))
    gpu = re.sub(r"/\*.*?\*/", "", open(os.path.join(INCLUDE, "sem2d_gpu.h")).read(), flags=re.S)
    declared = set(re.findall(r"\b(sem2d_gpu_\w+)\s*\(", gpu))
    assert bound == declared
    # constants with the header's values
    for m in re.finditer(r"#define\s+(SEM2D_\w+)\s+\(?(-?\d+)\)?\s", open(os.path.join(INCLUDE, "sem2d_gpu.h")).read()):
        assert re.search(r"parameter :: %s = %s\b" % (m.group(1), m.group(2)), src), m.group(1)


def test_version_and_errors_without_device():
    L = _lib.lib()
    assert L.sem2d_gpu_version() == 1
    # bad arguments are rejected before any device work
    h = C.c_void_p()
    assert L.sem2d_gpu_create(None, C.byref(h)) == abi.SEM2D_E_ARG
    assert b"null" in L.sem2d_gpu_last_error(None)
    assert L.sem2d_gpu_step(None, 1) == abi.SEM2D_E_ARG
