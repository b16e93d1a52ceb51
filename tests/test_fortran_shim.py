"""The ISO_C_BINDING shim aeroapps_gb300/fortran/aerort_mod.F90 binds only
entry points that include/aerort.h declares and the library exports, with the
C prototype's number of arguments, and every drop-in subroutine forwards the
reference routine's argument list (geo_vlidort/VLIDORT_LAMBERT.F90:34-37 and
:172-175, VLIDORT_ROT.F90:19, Chem_Base/MieObs_py.F90:27-28).  No Fortran
compiler is needed: the module is read as text."""
import ctypes
import os
import re

from aeroapps_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
F90 = os.path.join(ROOT, "aeroapps_gb300", "fortran", "aerort_mod.F90")


def _joined(src):
    src = "\n".join(ln.split("!")[0] for ln in src.splitlines())  # drop comments
    return re.sub(r"&\s*\n\s*", " ", src)                           # join continuation lines


def _c_prototypes():
    src = open(os.path.join(ROOT, "include", "aerort.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    out = {}
    for name, args in re.findall(r"\bint\s+(aerort_\w+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        out[name] = 0 if args.strip() in ("", "void") else args.count(",") + 1
    return out


def _bindings():
    src = _joined(open(F90).read())
    out = {}
    for args, cname in re.findall(r"function\s+\w+\s*\(([^)]*)\)\s*bind\(C,\s*name=\"(\w+)\"\)", src):
        out[cname] = 0 if not args.strip() else args.count(",") + 1
    return out


def _subroutine_args(name, src):
    m = re.search(r"subroutine\s+%s\s*\(([^)]*)\)" % name, _joined(src), flags=re.I)
    assert m, name
    return [a.strip().lower() for a in m.group(1).split(",")]


def test_bindings_match_header_and_exports():
    protos = _c_prototypes()
    binds = _bindings()
    assert len(binds) >= 9
    lib = ctypes.CDLL(build.build())
    for cname, nargs in binds.items():
        assert hasattr(lib, cname), cname
        if cname == "aerort_last_error":
            continue
        assert cname in protos, cname
        assert protos[cname] == nargs, (cname, protos[cname], nargs)


def test_drop_ins_keep_the_reference_argument_lists():
    shim = open(F90).read()
    ref_scalar = ("km nch nobs channels nstreams plane_parallel nmom npol rot depol tau ssa g pmom pe he te albedo "
                  "solar_zenith relat_azymuth sensor_zenith missing verbose radiance_vl reflectance_vl rc").split()
    ref_vector = ("km nch nobs channels nstreams plane_parallel nmom npol rot depol alpha tau ssa pmom pe he te albedo "
                  "solar_zenith relat_azymuth sensor_zenith flux_factor missing verbose radiance_vl reflectance_vl "
                  "q u rc").split()
    ref_rot = "km nch nobs channels pe he te missing verbose rot depol rc".split()
    ref_edge = "km nobs airdens delp ptop pe ze te rc".split()
    assert _subroutine_args("VLIDORT_Scalar_Lambert_GPU", shim) == ref_scalar
    assert _subroutine_args("VLIDORT_Vector_Lambert_GPU", shim) == ref_vector
    ref_modis = ("km nch nobs channels nstreams plane_parallel nmom npol rot depol tau ssa g pmom pe he te kernel_wt "
                 "param solar_zenith relat_azymuth sensor_zenith missing verbose radiance_vl_surf "
                 "reflectance_vl_surf br rc").split()
    assert _subroutine_args("VLIDORT_Scalar_LandMODIS_GPU", shim) == ref_modis
    # VLIDORT_Scalar_CX / _GissCX (VLIDORT_BRDF_CX.F90:420-423, :1553-1556)
    ref_cx = ("km nch nobs channels nstreams plane_parallel nmom npol rot depol tau ssa g pmom pe he te u10m v10m "
              "mr solar_zenith relat_azymuth sensor_zenith missing verbose radiance_vl_surf reflectance_vl_surf "
              "brdf rc").split()
    assert _subroutine_args("VLIDORT_Scalar_CX_GPU", shim) == ref_cx
    assert _subroutine_args("VLIDORT_Scalar_GissCX_GPU", shim) == ref_cx
    assert _subroutine_args("VLIDORT_ROT_CALC_GPU", shim) == ref_rot
    assert _subroutine_args("getEdgeVars_GPU", shim) == ref_edge
