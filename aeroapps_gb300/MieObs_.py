"""Drop-in for the f2py module MieObs_ (src/Shared/GMAO_Shared/Chem_Base/MieObs_py.F90)
with the work on the GPU.

Same function names (f2py lower-cases them), argument order and return
tuples as the calls in Chem_Base/mieobs.py:
  getmiedims(file)                                           -> (nCh, nRh, nBin, nMom, nPol, rc)
  getedgevars(airdens, delp, ptop)                            -> (pe, ze, te)
  getaopscalar(rcfile, channels, vname, verbose, qm, rh)      -> (tau, ssa, g, rc)
  getaopvector(rcfile, channels, vname, verbose, qm, rh, nMom, nPol) -> (tau, ssa, g, pmom, rc)
Array shapes are the Fortran ones: airdens/delp/rh (km, nobs), qm (km, nq,
nobs); vname is a list of names or an (nq, 16) character array.

The reference builds the Mie tables from the resource file on every call
(Chem_MieCreate ... Chem_MieDestroy, MieObs_py.F90:307-450); here the device
tables of a resource file stay resident between calls, keyed by its path and
modification time.  Tracer names follow the registry Chem_MieCreateFromRC
reads from the working directory (Chem_MieRegistry.rc, else
Chem_Registry.rc; Chem_MieMod.F90:174-181); without either, a tracer is
<table name><bin, 3 digits>.  getext and getint (lidar extinction and
backscatter, MieObs_py.F90:460-770) are off the radiance path and not
provided.
"""
import os

import numpy as np

from . import mie

_cache = {}


def _stamp(path):
    try:
        return os.path.abspath(path), os.path.getmtime(path)
    except OSError:
        return os.path.abspath(path), None


def _registry_file():
    for name in ("Chem_MieRegistry.rc", "Chem_Registry.rc"):
        if os.path.exists(name):
            return name
    return None


def _names(vname):
    """Tracer names from f2py-style input: strings (padded to 16) or an
    (nq, 16) array of characters."""
    a = np.asarray(vname)
    if a.ndim == 2:
        rows = ["".join(x.decode() if isinstance(x, bytes) else str(x) for x in row) for row in a]
    else:
        rows = [x.decode() if isinstance(x, bytes) else str(x) for x in a.ravel()]
    return [r.strip() for r in rows]


def _chem(rcfile):
    reg_file = _registry_file()
    key = (_stamp(rcfile), _stamp(reg_file) if reg_file else None)
    chem = _cache.get(key)
    if chem is None:
        tables = mie.tables_from_rc(rcfile)
        registry = None
        if reg_file:
            registry = mie.registry_map(mie.read_chem_registry(reg_file), [t.name for t in tables.tables])
        chem = mie.ChemMie(tables, registry=registry)
        for k in [k for k in _cache if k[0][0] == key[0][0]]:
            _cache.pop(k).destroy()
        _cache[key] = chem
    return chem


def getmiedims(file):
    return mie.get_mie_dims(file)


def getedgevars(airdens, delp, ptop):
    airdens = np.asarray(airdens)
    km, nobs = airdens.shape
    return mie.get_edge_vars(km, nobs, airdens, delp, ptop)


def getaopscalar(rcfile, channels, vname, verbose, qm, rh):
    names = _names(vname)
    qm = np.asarray(qm)
    km, nq, nobs = qm.shape
    ch = np.atleast_1d(np.asarray(channels, np.float32))
    return mie.get_aop_scalar(_chem(rcfile), km, nobs, len(ch), nq, ch, names, int(verbose), qm, rh)


def getaopvector(rcfile, channels, vname, verbose, qm, rh, nMom, nPol):
    names = _names(vname)
    qm = np.asarray(qm)
    km, nq, nobs = qm.shape
    ch = np.atleast_1d(np.asarray(channels, np.float32))
    return mie.get_aop_vector(_chem(rcfile), km, nobs, len(ch), nq, ch, names, int(verbose), qm, rh, int(nMom),
                              int(nPol))
