"""netCDF-4 (HDF5) optics tables: aeroapps_gb300/nc4.py, the read-only HDF5
reader behind mie.read_optics_file and mie.get_mie_dims for the netCDF-4
files that Chem_MieTableRead opens with the netCDF library
(Chem_MieTableMod.F90:297-466, Chem_MieTableGetDims :733-800).

- A netCDF-4 file written by the netCDF/HDF5 libraries: the reference tree's
  PACE f/Q table (superblock 2, dense links in a fractal heap with a
  version-2 B-tree name index, dimension scales with and without coordinate
  variables, DIMENSION_LIST references in the global heap); skipped where
  that tree is absent.
- Files of tests/nc4_writer.py (the same structures, written here): every
  chunk index (version-1 B-tree, fixed array, single chunk, implicit) with
  and without the shuffle and deflate filters, edge chunks included, and the
  older layout (superblock 0, version-1 object headers, symbol-table group),
  read back bit for bit; an optics table read from netCDF-4 equal to the same
  table read from netCDF classic."""
import os

import numpy as np
import pytest

from aeroapps_gb300 import mie, nc4

import nc4_writer
from test_mie_read import _raw_table, _write_nc

REF_FQ = os.path.join(os.environ.get("AEROAPPS_REFERENCE", "/root/reference"),
                      "src/Components/missions/PACE/oci_tables/morel_fq.nc")


@pytest.mark.skipif(not os.path.exists(REF_FQ), reason="reference tree absent")
def test_reads_a_library_written_netcdf4_file():
    ds = nc4.Dataset(REF_FQ)
    assert ds.dimensions == {"n_wave": 7, "n_solz": 6, "n_chl": 6, "n_senz": 17, "n_phi": 13}
    v = ds.variables
    assert set(v) == {"wave", "solz", "chl", "senz", "phi", "foq"}
    assert v["foq"].dimensions == ("n_wave", "n_solz", "n_chl", "n_senz", "n_phi")
    assert v["solz"].dimensions == ("n_solz",) and v["solz"].attributes["units"] == "degrees"
    assert np.array_equal(v["solz"].values(), np.arange(0, 76, 15, dtype=np.float32))
    assert np.array_equal(v["phi"].values(), np.arange(0, 181, 15, dtype=np.float32))
    assert np.array_equal(v["wave"].values(), np.array([412.5, 442.5, 490, 510, 560, 620, 660], np.float32))
    assert np.allclose(v["chl"].values(), [0.03, 0.1, 0.3, 1.0, 3.0, 10.0])
    senz = v["senz"].values()
    assert senz.shape == (17,) and np.all(np.diff(senz) > 0)
    foq = v["foq"].values()
    # f/Q of the Morel tables: a ratio of order 0.1 everywhere
    assert foq.shape == (7, 6, 6, 17, 13) and foq.dtype == np.float32
    assert np.all(np.isfinite(foq)) and 0.05 < foq.min() and foq.max() < 0.5


@pytest.mark.parametrize("index,shuffle,deflate,legacy", [("btree1", True, True, False), ("btree1", False, False, False),
                                                          ("farray", True, True, False), ("farray", False, True, False),
                                                          ("single", True, True, False), ("implicit", False, False, False),
                                                          ("btree1", True, True, True), ("btree1", False, True, True)])
def test_chunk_indexes_and_filters_round_trip(tmp_path, index, shuffle, deflate, legacy):
    # legacy: superblock 0, version-1 object headers, attributes and filter
    # pipeline, the root group as a symbol table
    r = np.random.default_rng(3)
    a = r.normal(size=(5, 7, 3))
    path = os.path.join(tmp_path, "t.nc")
    chunk = (lambda s: s) if index == "single" else (lambda s: (2, 3, 2))  # ragged edge chunks
    nc4_writer.write(path, [("x", 5, np.arange(5.0)), ("y", 7, None), ("z", 3, None)],
                     [("a", ("x", "y", "z"), a), ("b", ("z", "x", "y"), np.transpose(a, (2, 0, 1)))],
                     index=index, chunk=chunk, shuffle=shuffle, deflate=deflate, legacy=legacy)
    ds = nc4.Dataset(path)
    assert ds.dimensions == {"x": 5, "y": 7, "z": 3}
    assert set(ds.variables) == {"x", "a", "b"}
    assert ds.variables["a"].dimensions == ("x", "y", "z")
    assert ds.variables["b"].dimensions == ("z", "x", "y")
    assert np.array_equal(ds.variables["a"].values(), a)
    assert np.array_equal(ds.variables["b"].values(), np.transpose(a, (2, 0, 1)))
    assert np.array_equal(ds.variables["x"].values(), np.arange(5.0))


def _write_nc4(path, t, index="btree1"):
    """The optics table of test_mie_read._raw_table as netCDF-4, C-order
    dimensions (nPol, nMom, radius, rh, lambda) as a Fortran writer declares
    them; lambda and rh are coordinate variables."""
    nlam, nrh, nbin, nmom, npol = t["pmom"].shape
    dims = [("lambda", nlam, t["lam"]), ("rh", nrh, t["rh"]), ("radius", nbin, None), ("nMom", nmom, None),
            ("nPol", npol, None)]
    c3 = ("radius", "rh", "lambda")
    var = [(n, c3, np.transpose(t[n])) for n in ("bext", "bsca", "g")]
    var.append(("pmom", ("nPol", "nMom") + c3, np.transpose(t["pmom"])))
    nc4_writer.write(path, dims, var, index=index)


@pytest.mark.parametrize("index", ["btree1", "farray"])
def test_optics_table_from_netcdf4_equals_netcdf_classic(tmp_path, index):
    t = _raw_table(11)
    p3, p4 = os.path.join(tmp_path, "optics_c.nc"), os.path.join(tmp_path, "optics_4.nc")
    _write_nc(p3, t)
    _write_nc4(p4, t, index)
    a, b = mie.read_optics_file(p3), mie.read_optics_file(p4)
    for k in ("lambda", "rh", "bext", "bsca", "g", "pmom"):
        assert np.array_equal(a[k], b[k]), k
    assert mie.get_mie_dims(p4) == mie.get_mie_dims(p3) == (10, 6, 4, 9, 2, 0)


def test_unreadable_hdf5_file(tmp_path):
    path = os.path.join(tmp_path, "optics_h5.nc")
    with open(path, "wb") as fh:
        fh.write(nc4.MAGIC + bytes(64))
    with pytest.raises(ValueError):
        mie.read_optics_file(path)
    assert mie.get_mie_dims(path) == (0, 0, 0, 0, 0, 1)
