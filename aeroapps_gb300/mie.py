"""Mie tables (Chem_Mie) and the aerosol-optics mixing (VLIDORT_getAOPvector).

Mirrors the reference interface of
  src/Shared/GMAO_Shared/Chem_Base/Chem_MieMod.F90      (Chem_MieCreate, Chem_MieQueryIdx,
                                                         Chem_MieQuery, Chem_MieDestroy)
  src/Components/rtms/geo_vlidort/VLIDORT_MieMod.F90    (VLIDORT_getAOPvector)
with the tables held on the GPU.  Table data come either from GEOS
optics_*.nc files (`read_tables`: the netCDF read and the wavelength
interpolation of Chem_MieTableRead, Chem_MieTableMod.F90:238-719) or from
`generate_tables` (a Lorenz-Mie series over lognormal size distributions).
"""
import ctypes
import dataclasses
import hashlib
import os

import numpy as np

from . import _lib, nc4

# Five GOCART-like species: name prefix, refractive index (n, k) of the dry
# aerosol, dry density [kg m-3], hygroscopic growth (dust does not grow).
SPECIES = [
    ("su", 1.43, 0.0, 1700.0, True),      # sulfate
    ("du", 1.53, 0.003, 2650.0, False),   # dust
    ("ss", 1.50, 1.0e-8, 2200.0, True),   # sea salt
    ("oc", 1.53, 0.006, 1800.0, True),    # organic carbon
    ("bc", 1.75, 0.44, 1000.0, True),     # black carbon
]
NBIN = 4
# dry number-mode radius and geometric width of the 4 size bins: log-spaced
# 0.05..1.0 um, sigma_g 1.6..2.0
BIN_RG_UM = tuple(0.05 * 20.0 ** (b / 3.0) for b in range(NBIN))
BIN_SIGMA = tuple(1.6 + 0.4 * b / 3.0 for b in range(NBIN))
NRH = 36


@dataclasses.dataclass
class MieTable:
    """One species table in Chem_MieTable layout (Fortran order, REAL*4)."""
    name: str
    rh: np.ndarray      # (nrh,)
    bext: np.ndarray    # (nrh, nch, nbin)
    bsca: np.ndarray
    g: np.ndarray
    pmom: np.ndarray    # (nrh, nch, nbin, nmom, npol)


@dataclasses.dataclass
class MieTableSet:
    channels_m: np.ndarray  # (nch,) wavelengths [m]
    tables: list

    def tracer_names(self):
        return ["%s%03d" % (t.name, b + 1) for t in self.tables for b in range(t.bext.shape[2])]


def _cache_dir():
    d = os.environ.get("AERORT_CACHE")
    if d:
        return d
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "mie_cache")


def generate_tables(channels_nm, nmom=64, nrh=NRH, nradii=160, use_cache=True, npol=1):
    """Synthetic GEOS-style Mie tables at the requested channels [nm].

    RH nodes: nrh values evenly spaced on [0, 0.99] (REAL*4).  Wet particles:
    radius x (1-RH)^-0.2, refractive index volume-mixed with water.  npol = 1:
    P11 Legendre moments; npol = 6: the Greek coefficients of P11, P12, P33,
    P34, P22, P44 (the layout of the GEOS optics tables used by the polarized
    path).
    """
    if npol not in (1, 6):
        raise ValueError("npol must be 1 or 6")
    channels_nm = np.asarray(channels_nm, dtype=np.float64)
    ident = (channels_nm.tolist(), nmom, nrh, nradii, SPECIES, BIN_RG_UM, BIN_SIGMA, "quad512")
    if npol != 1:
        ident = ident + (npol,)
    key = hashlib.sha256(repr(ident).encode()).hexdigest()[:16]
    path = os.path.join(_cache_dir(), "mie_%s.npz" % key)
    rh = np.linspace(0.0, 0.99, nrh).astype(np.float32)
    if use_cache and os.path.exists(path):
        z = np.load(path)
        tabs = []
        for s in SPECIES:
            n = s[0]
            tabs.append(MieTable(n, rh, np.asfortranarray(z[n + "_bext"]), np.asfortranarray(z[n + "_bsca"]),
                                 np.asfortranarray(z[n + "_g"]), np.asfortranarray(z[n + "_pmom"])))
        return MieTableSet((channels_nm * 1e-9).astype(np.float32), tabs)
    L = _lib.lib()
    nch = len(channels_nm)
    lam = np.ascontiguousarray(channels_nm * 1e-3)
    rh64 = rh.astype(np.float64)
    rg = np.array(BIN_RG_UM)
    sg = np.array(BIN_SIGMA)
    tabs = []
    save = {}
    for (name, nr, ni, rho, hyg) in SPECIES:
        bext = np.zeros((nrh, nch, NBIN), np.float32, order="F")
        bsca = np.zeros_like(bext)
        g = np.zeros_like(bext)
        pm = np.zeros((nrh, nch, NBIN, nmom, npol), np.float32, order="F")
        rc = L.aerort_miegen_lognormal_pol(nch, _lib.ptr(lam, _lib.P_d), nrh, _lib.ptr(rh64, _lib.P_d), NBIN,
                                           _lib.ptr(rg, _lib.P_d), _lib.ptr(sg, _lib.P_d), nr, ni, int(hyg), rho, nmom,
                                           npol, nradii, _lib.ptr(bext, _lib.P_f), _lib.ptr(bsca, _lib.P_f),
                                           _lib.ptr(g, _lib.P_f), _lib.ptr(pm, _lib.P_f))
        if rc != 0:
            raise RuntimeError("Mie table generation failed for %s" % name)
        tabs.append(MieTable(name, rh, bext, bsca, g, pm))
        save.update({name + "_bext": bext, name + "_bsca": bsca, name + "_g": g, name + "_pmom": pm})
    if use_cache:
        os.makedirs(_cache_dir(), exist_ok=True)
        tmp = path + ".tmp.npz"
        np.savez(tmp, **save)
        os.replace(tmp, path)
    return MieTableSet((channels_nm * 1e-9).astype(np.float32), tabs)


_HDF5_MAGIC = b"\x89HDF\r\n\x1a\n"
_FIELDS3 = ("lambda", "rh", "radius")
_FIELDS5 = ("lambda", "rh", "radius", "nMom", "nPol")


class _OpticsFile:
    """dimensions {name: length} and variables {name: (dimension names, loader)}
    of one optics file, netCDF classic / 64-bit offset (scipy) or netCDF-4
    (HDF5, nc4.Dataset)."""

    def __init__(self, path):
        with open(path, "rb") as fh:
            hdf5 = fh.read(8) == _HDF5_MAGIC
        if hdf5:
            nc = nc4.Dataset(path)
            self.dimensions = dict(nc.dimensions)
            self.variables = {n: (tuple(v.dimensions), v.values) for n, v in nc.variables.items()}
            return
        from scipy.io import netcdf_file
        with netcdf_file(path, "r", mmap=False) as nc:
            self.dimensions = {n: int(x) for n, x in nc.dimensions.items() if x is not None}
            data = {n: (tuple(v.dimensions), np.array(v.data)) for n, v in nc.variables.items()}
        self.variables = {n: (dims, (lambda a=a: a)) for n, (dims, a) in data.items()}


def read_optics_file(path):
    """The arrays Chem_MieTableRead reads from one optics_*.nc file
    (Chem_MieTableMod.F90:297-466): lambda [m], rh, and bext, bsca, g
    (nlambda, nrh, nbin) and pmom (nlambda, nrh, nbin, nMom, nPol) as REAL*8,
    axes ordered by dimension name whatever the file's declaration order
    (pmom None when the file has none).  Values are taken as stored, without
    scale/offset attributes, as nf_get_var_double does.

    Reads netCDF classic and 64-bit-offset files (scipy) and netCDF-4 files
    (HDF5: nc4.py)."""
    f = _OpticsFile(path)
    v = f.variables

    def arr(name, order):
        dims, load = v[name]
        if sorted(dims) != sorted(order):
            raise ValueError("%s: variable %s has dimensions %s, expected %s" % (path, name, dims, order))
        a = np.asarray(load(), np.float64)
        return np.asfortranarray(np.transpose(a, [dims.index(d) for d in order]))

    out = {"lambda": np.asarray(v["lambda"][1](), np.float64).ravel().copy(),
           "rh": np.asarray(v["rh"][1](), np.float64).ravel().copy()}
    for name in ("bext", "bsca", "g"):
        out[name] = arr(name, _FIELDS3)
    out["pmom"] = arr("pmom", _FIELDS5) if "pmom" in v else None
    return out


def get_mie_dims(path):
    """getMieDims / Chem_MieTableGetDims (MieObs_py.F90:7-23,
    Chem_MieTableMod.F90:733-800): (nCh, nRh, nBin, nMom, nPol, rc) of one
    optics file (netCDF classic or netCDF-4).  A file without an nMom
    dimension has nMom = nPol = 0, as in the reference.  rc is nonzero, with
    zero sizes, when the file or one of the lambda/rh/radius dimensions
    cannot be read."""
    try:
        d = _OpticsFile(path).dimensions
        nch, nrh, nbin = int(d["lambda"]), int(d["rh"]), int(d["radius"])
        nmom = int(d["nMom"]) if "nMom" in d else 0
        npol = int(d["nPol"]) if "nMom" in d and "nPol" in d else 0
        return nch, nrh, nbin, nmom, npol, 0
    except (OSError, KeyError, TypeError, ValueError):
        return 0, 0, 0, 0, 0, 1


def table_from_file_arrays(name, lam, rh, bext, bsca, g, pmom, channels_m, nmom):
    """Chem_MieTableRead's set-up of one table (Chem_MieTableMod.F90:557-601):
    the file arrays (wavelength first, REAL*8) interpolated to channels_m [m]
    with the reference's polint, through aerort_mie_table_interp.  Returns
    (MieTable, number of channels outside the table's wavelength range)."""
    f = lambda a: np.asfortranarray(a, np.float64)
    lam = np.ascontiguousarray(lam, np.float64)
    rh = np.ascontiguousarray(rh, np.float64)
    bext, bsca, g = f(bext), f(bsca), f(g)
    nlam, nrh, nbin = bext.shape
    if pmom is None:
        if nmom > 0:
            raise ValueError("table %s has no pmom, %d moments requested" % (name, nmom))
        pmom = np.zeros((nlam, nrh, nbin, 0, 1))
    pmom = f(pmom)
    nmom_table, npol = pmom.shape[3], pmom.shape[4]
    ch = np.ascontiguousarray(channels_m, np.float32)
    nch = len(ch)
    orh = np.zeros(nrh, np.float32)
    ob = [np.zeros((nrh, nch, nbin), np.float32, order="F") for _ in range(3)]
    opm = np.zeros((nrh, nch, nbin, nmom, npol), np.float32, order="F")
    nout = ctypes.c_int(0)
    rc = _lib.lib().aerort_mie_table_interp(
        nlam, _lib.ptr(lam, _lib.P_d), nrh, _lib.ptr(rh, _lib.P_d), nbin, nmom_table, npol,
        _lib.ptr(bext, _lib.P_d), _lib.ptr(bsca, _lib.P_d), _lib.ptr(g, _lib.P_d),
        _lib.ptr(pmom, _lib.P_d) if pmom.size else None, nch, _lib.ptr(ch, _lib.P_f), nmom,
        _lib.ptr(orh, _lib.P_f), *[_lib.ptr(a, _lib.P_f) for a in ob], _lib.ptr(opm, _lib.P_f) if opm.size else None,
        ctypes.byref(nout))
    if rc != 0:
        raise RuntimeError("aerort_mie_table_interp rc=%d for table %s (nmom %d, table has %d)"
                           % (rc, name, nmom, nmom_table))
    return MieTable(name, orh, ob[0], ob[1], ob[2], opm), nout.value


def read_tables(files, channels_nm, nmom, channels_m=None):
    """Chem_MieCreate's table reads (Chem_MieMod.F90:326-339): one optics file
    per species, {name: path} in table order, each interpolated to the
    channels [nm] (or to channels_m [m], REAL*4, when given).  Channels outside
    a table's wavelength range are allowed, as in the reference, and reported
    through warnings.warn."""
    import warnings
    if channels_m is not None:
        ch = np.ascontiguousarray(channels_m, np.float32)
    else:
        ch = (np.asarray(channels_nm, np.float64) * 1e-9).astype(np.float32)
    tabs = []
    for name, path in files.items():
        a = read_optics_file(path)
        t, nout = table_from_file_arrays(name, a["lambda"], a["rh"], a["bext"], a["bsca"], a["g"], a["pmom"], ch, nmom)
        if nout:
            warnings.warn("Mie table %s (%s): %d channel(s) outside its wavelength range %g..%g m"
                          % (name, path, nout, a["lambda"][0], a["lambda"][-1]))
        tabs.append(t)
    return MieTableSet(ch, tabs)


# species of a Mie resource file, in Chem_MieCreate's table-read order (Chem_MieMod.F90:326-339)
RC_SPECIES = ("du", "ss", "su", "oc", "bc", "ni", "brc")


def read_mie_rc(rcfile):
    """The Mie resource file of Chem_MieCreateFromRC (Chem_MieMod.F90:124-300):
    n_channels, optional n_moments (default 0), r_channels [m] and
    filename_optical_properties_<DU|SS|BC|OC|SU|NI|BRC>.  Lines are
    `label: values`; `#` starts a comment.  Returns {"nch", "nmom",
    "channels_m" (REAL*4), "files": {species: path}}.  A relative table
    path is opened from the working directory, as nf_open does in the
    reference; when no such file is there, from the resource file's
    directory.  Raises ValueError where the reference stops (missing or
    unparsable entries)."""
    entries = {}
    with open(rcfile) as f:
        for line in f:
            line = line.split("#", 1)[0].strip()
            if ":" not in line:
                continue
            label, rest = line.split(":", 1)
            entries[label.strip()] = rest.split()

    def need(label):
        if label not in entries or not entries[label]:
            raise ValueError("%s: could not find %s" % (rcfile, label))
        return entries[label]

    try:
        nch = int(need("n_channels")[0])
        nmom = int(entries["n_moments"][0]) if entries.get("n_moments") else 0
        chans = need("r_channels")
        if len(chans) < nch:
            raise ValueError("%s: r_channels has %d values, n_channels is %d" % (rcfile, len(chans), nch))
        ch = np.array([float(x.replace("d", "e").replace("D", "e")) for x in chans[:nch]], np.float32)
    except (ValueError, IndexError) as e:
        raise ValueError("%s: could not parse channels or moments (%s)" % (rcfile, e))
    base = os.path.dirname(os.path.abspath(rcfile))
    files = {}
    for sp in RC_SPECIES:
        path = need("filename_optical_properties_%s" % sp.upper())[0]
        if not os.path.isabs(path):
            path = os.path.abspath(path) if os.path.exists(path) else os.path.join(base, path)
        files[sp] = path
    return {"nch": nch, "nmom": nmom, "channels_m": ch, "files": files}


def tables_from_rc(rcfile):
    """Every table of a Mie resource file, read and interpolated to its
    channels with its moment count (Chem_MieCreateFromRC + Chem_MieTableRead)."""
    rc = read_mie_rc(rcfile)
    return read_tables(rc["files"], None, rc["nmom"], channels_m=rc["channels_m"])


def read_chem_registry(path):
    """The aerosol part of Chem_RegistryCreate (Chem_RegistryMod.F90:185-552)
    as Chem_MieCreate uses it: for each of du, ss, su, bc, oc, brc, ni with
    `doing_XX: y...` and `nbins_XX` >= 1, the tracer names in registry order.
    Names come from the first nbins lines of a `variable_table_XX::` block
    (first token of each line) when there is one, else <species><bin, 3
    digits>.  Returns {species: [names]} for registry_map."""
    lines = []
    with open(path) as f:
        for line in f:
            lines.append(line.split("#", 1)[0].rstrip("\n"))

    def value(label):
        for ln in lines:
            t = ln.strip()
            if t.startswith(label):
                rest = t[len(label):].split()
                return rest[0] if rest else None
        return None

    groups = {}
    for sp in ("du", "ss", "su", "bc", "oc", "brc", "ni"):
        doing = value("doing_%s:" % sp.upper())
        if not doing or doing[0] not in "yY":
            continue
        nb = value("nbins_%s:" % sp.upper())
        if nb is None:
            raise ValueError("%s: cannot determine NBINS for %s" % (path, sp.upper()))
        nbins = int(nb)
        if nbins < 1:
            continue
        names = None
        token = "variable_table_%s::" % sp.upper()
        for i, ln in enumerate(lines):
            if ln.strip().startswith(token):
                names = []
                for row in lines[i + 1:]:
                    tok = row.split()
                    if not tok:
                        continue
                    if tok[0] == "::" or len(names) == nbins:
                        break
                    names.append(tok[0])
                if len(names) < nbins:
                    raise ValueError("%s: not enough names in %s" % (path, token))
                break
        groups[sp] = names if names is not None else ["%s%03d" % (sp, b + 1) for b in range(nbins)]
    return groups


def registry_map(groups, tables):
    """The tracer -> (table, bin) hash of Chem_MieCreate (Chem_MieMod.F90:345-399).

    groups: {species: [tracer names in registry order]} with species among
    du, ss, oc, brc, bc, su, ni; tables: the table names in table order.
    du/ss/oc/brc/bc tracers take bins 1, 2, ... in registry order; for su only
    the names beginning so4/SO4/sul/SUL, and for ni only no3/NO3, count, the
    others keep no optics.  Returns {upper-case name: (table index, 0-based
    bin)}; unmapped names are absent."""
    out = {}
    for sp, names in groups.items():
        ti = tables.index(sp)
        if sp in ("du", "ss", "oc", "brc", "bc"):
            for b, n in enumerate(names):
                out[n.strip().upper()] = (ti, b)
        elif sp in ("su", "ni"):
            keys = ("so4", "SO4", "sul", "SUL") if sp == "su" else ("no3", "NO3")
            b = 0
            for n in names:
                if n.strip()[:3] in keys:
                    out[n.strip().upper()] = (ti, b)
                    b += 1
        else:
            raise ValueError("unknown species group %r" % sp)
    return out


class ChemMie:
    """Device-resident Chem_Mie object (Chem_MieMod.F90:41-47).

    registry: optional {upper-case tracer name: (table, bin)} as made by
    registry_map; without it tracer names are <table name><bin, 3 digits>."""

    def __init__(self, tableset, registry=None):
        self.tableset = tableset
        self.registry = registry
        self.names = [t.name for t in tableset.tables]
        descs = (_lib.MieTableDesc * len(tableset.tables))()
        self._keep = []
        for i, t in enumerate(tableset.tables):
            arrs = [np.asfortranarray(t.rh, np.float32), np.asfortranarray(t.bext, np.float32),
                    np.asfortranarray(t.bsca, np.float32), np.asfortranarray(t.g, np.float32),
                    np.asfortranarray(t.pmom, np.float32)]
            self._keep += arrs
            descs[i].nrh = t.rh.shape[0]
            descs[i].nbin = t.bext.shape[2]
            descs[i].nmom = t.pmom.shape[3]
            descs[i].npol = t.pmom.shape[4]
            descs[i].rh, descs[i].bext, descs[i].bsca, descs[i].g, descs[i].pmom = [_lib.ptr(a, _lib.P_f) for a in arrs]
        ch = np.ascontiguousarray(tableset.channels_m, np.float32)
        h = ctypes.c_void_p()
        rc = _lib.lib().aerort_mie_create(len(tableset.tables), descs, len(ch), _lib.ptr(ch, _lib.P_f), ctypes.byref(h))
        if rc != 0:
            raise RuntimeError("aerort_mie_create rc=%d: %s" % (rc, _lib.last_error()))
        self.handle = h
        self.channels = ch

    @classmethod
    def from_rc(cls, rcfile, registry=None):
        """Chem_MieCreate(rcfile) (Chem_MieMod.F90:124-411) on the device."""
        return cls(tables_from_rc(rcfile), registry=registry)

    def query_idx(self, vname):
        """Chem_MieQueryIdx (Chem_MieMod.F90:720-777): tracer name -> (table, bin) or (-1, -1).
        Case-insensitive; a qualifier such as GOCART:: is dropped (:750-754)."""
        v = vname.strip()
        i = v.find("::")
        if i >= 0:
            v = v[i + 2:]
        if self.registry is not None:
            return self.registry.get(v.strip().upper(), (-1, -1))
        v = v.strip().lower()
        for ti, t in enumerate(self.tableset.tables):
            for b in range(t.bext.shape[2]):
                if v == "%s%03d" % (t.name, b + 1):
                    return ti, b
        return -1, -1

    def destroy(self):
        if self.handle:
            _lib.lib().aerort_mie_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


def get_aop_vector(mie, km, nobs, nch, nq, channels, vname, verbose, qm, rh, nMom, nPol):
    """VLIDORT_getAOPvector (VLIDORT_MieMod.F90:124-336).

    Returns (tau, ssa, g, pmom, rc) with the reference shapes
    tau/ssa/g (km,nch,nobs), pmom (km,nch,nobs,nMom,nPol), FP32, Fortran order.
    """
    qtab = np.empty(nq, np.int32)
    qbin = np.empty(nq, np.int32)
    for iq in range(nq):
        qtab[iq], qbin[iq] = mie.query_idx(vname[iq])
    ch = np.ascontiguousarray(channels, np.float32)
    qm = np.asfortranarray(qm, np.float32)
    rh = np.asfortranarray(rh, np.float32)
    tau = np.zeros((km, nch, nobs), np.float32, order="F")
    ssa = np.zeros_like(tau)
    g = np.zeros_like(tau)
    pmom = np.zeros((km, nch, nobs, nMom, nPol), np.float32, order="F")
    rc = _lib.lib().aerort_get_aop_vector(mie.handle, km, nobs, nch, nq, _lib.ptr(ch, _lib.P_f), _lib.ptr(qtab, _lib.P_i),
                                          _lib.ptr(qbin, _lib.P_i), _lib.ptr(qm, _lib.P_f), _lib.ptr(rh, _lib.P_f),
                                          nMom, nPol, _lib.ptr(tau, _lib.P_f), _lib.ptr(ssa, _lib.P_f),
                                          _lib.ptr(g, _lib.P_f), _lib.ptr(pmom, _lib.P_f))
    if rc not in (0, 99, 666, 777):
        raise RuntimeError("aerort_get_aop_vector rc=%d: %s" % (rc, _lib.last_error()))
    return tau, ssa, g, pmom, rc


def get_aop_scalar(mie, km, nobs, nch, nq, channels, vname, verbose, qm, rh):
    """VLIDORT_getAOPscalar (VLIDORT_MieMod.F90:10-120).

    Returns (tau, ssa, g, rc), each (km,nch,nobs), FP32, Fortran order."""
    qtab = np.empty(nq, np.int32)
    qbin = np.empty(nq, np.int32)
    for iq in range(nq):
        qtab[iq], qbin[iq] = mie.query_idx(vname[iq])
    ch = np.ascontiguousarray(channels, np.float32)
    qm = np.asfortranarray(qm, np.float32)
    rh = np.asfortranarray(rh, np.float32)
    tau = np.zeros((km, nch, nobs), np.float32, order="F")
    ssa = np.zeros_like(tau)
    g = np.zeros_like(tau)
    rc = _lib.lib().aerort_get_aop_scalar(mie.handle, km, nobs, nch, nq, _lib.ptr(ch, _lib.P_f), _lib.ptr(qtab, _lib.P_i),
                                          _lib.ptr(qbin, _lib.P_i), _lib.ptr(qm, _lib.P_f), _lib.ptr(rh, _lib.P_f),
                                          _lib.ptr(tau, _lib.P_f), _lib.ptr(ssa, _lib.P_f), _lib.ptr(g, _lib.P_f))
    if rc not in (0, 99):
        raise RuntimeError("aerort_get_aop_scalar rc=%d: %s" % (rc, _lib.last_error()))
    return tau, ssa, g, rc


def get_edge_vars(km, nobs, airdens, delp, ptop):
    """getEdgeVars (MieObs_py.F90:27-83) on the GPU: edge pressure [Pa],
    height above the surface [m] and temperature [K], each (km+1, nobs) REAL*4,
    from airdens and delp (km, nobs) and the top pressure ptop [Pa].
    Returns (pe, ze, te) like the f2py routine."""
    rho = np.asfortranarray(airdens, np.float32)
    dp = np.asfortranarray(delp, np.float32)
    if rho.shape != (km, nobs) or dp.shape != (km, nobs):
        raise ValueError("airdens and delp must be (km, nobs) = (%d, %d)" % (km, nobs))
    pe, ze, te = [np.zeros((km + 1, nobs), np.float32, order="F") for _ in range(3)]
    rc = _lib.lib().aerort_get_edge_vars(km, nobs, _lib.ptr(rho, _lib.P_f), _lib.ptr(dp, _lib.P_f), float(ptop),
                                         _lib.ptr(pe, _lib.P_f), _lib.ptr(ze, _lib.P_f), _lib.ptr(te, _lib.P_f))
    if rc != 0:
        raise RuntimeError("aerort_get_edge_vars rc=%d: %s" % (rc, _lib.last_error()))
    return pe, ze, te
