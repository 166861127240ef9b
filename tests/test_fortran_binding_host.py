"""Static checks of the Fortran ISO_C_BINDING module (acumen_gb300/fortran/
acumen_gpu.f90).  No Fortran compiler exists in this image or on the GPU
hosts, so the module is checked against the C header as text: every bind(C)
interface names an entry point the header declares, with the same number of
arguments, passing by value exactly the header's scalar parameters; and the
drop-in module's ensure_ctx rebuilds the library context whenever the grid,
the angles or the mask taper change (a driver may change theta, nimage or wpu
between calls at the same ntheta)."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "acumen_gb300", "fortran", "acumen_gpu.f90")


def c_prototypes():
    txt = "".join(open(h).read() for h in glob.glob(os.path.join(ROOT, "include", "*.h")))
    txt = re.sub(r"/\*.*?\*/", " ", txt, flags=re.S)
    protos = {}
    for m in re.finditer(r"(?:int|const char \*)\s*(acu_\w+)\s*\(([^)]*)\)\s*;", txt):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        protos[m.group(1)] = params
    return protos


def f90_interfaces():
    src = open(F90).read().replace("&\n", " ")
    out = {}
    for m in re.finditer(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)(.*?)end function", src,
                         re.S | re.I):
        args = [a.strip() for a in m.group(2).split(",") if a.strip()]
        body = m.group(4)
        by_value = set()
        for decl in re.finditer(r"^\s*([^!\n]*?),\s*value\s*::\s*([^\n!]+)", body, re.M | re.I):
            by_value |= {v.strip() for v in decl.group(2).split(",")}
        out[m.group(3)] = (args, by_value)
    return out


def test_every_bind_c_interface_matches_the_header():
    protos = c_prototypes()
    ifaces = f90_interfaces()
    assert len(ifaces) >= 8
    for name, (args, by_value) in ifaces.items():
        assert name in protos, name
        params = protos[name]
        assert len(args) == len(params), (name, args, params)
        for a, p in zip(args, params):
            c_scalar = "*" not in p
            # a C pointer is a Fortran array, an intent(out) scalar, or a c_ptr passed by value;
            # a C scalar must be passed by value
            if c_scalar:
                assert a in by_value, (name, a, p)


def test_ensure_ctx_rebuilds_on_any_geometry_change():
    src = open(F90).read()
    body = re.search(r"subroutine ensure_ctx\(\)(.*?)end subroutine ensure_ctx", src, re.S).group(1)
    cond = body[:body.index("if (same) return")]
    for v in ("ctx_nimage == nimage", "ctx_ntheta == ntheta", "ctx_wpu == wpu", "ctx_theta == theta(1:ntheta)"):
        assert v in cond, v
    for v in ("ctx_nimage = nimage", "ctx_ntheta = ntheta", "ctx_wpu = wpu", "ctx_theta = theta(1:ntheta)"):
        assert v in body, v
    fin = re.search(r"subroutine fin_radon\(\)(.*?)end subroutine fin_radon", src, re.S).group(1)
    assert "ctx_ntheta = -1" in fin
