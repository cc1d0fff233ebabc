"""The reference's own outputs, as committed fixtures (tests/golden/, made by
tests/golden/make_reference_golden.py from the reference's CUDA build on a
GPU), checked on the CPU.

* one_thread_* (2D) and one_thread_3d_*: a one-thread run of the
  reference's sweep is an ordinary sequential Cellular Potts run driven by
  its Park-Miller generator.  tests/refmodel.py must reproduce the
  reference's lattice and its area and perimeter tables bit for bit from the
  stored inputs.  refmodel's dH is the one test_oracle.py replays against
  the oracle (2D and 3D), which pins the oracle's energy to the reference's
  outputs.
* recount_* (and the tables before every one-thread run): the oracle's
  table recount equals the reference's calculateAreasAndCircumferences
  tables (src/kernels2d.cu:5-41, src/kernels3d.cu:3-47).
"""
import pathlib

import numpy as np
import pytest

import oracle
import refmodel

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
ONE_THREAD = sorted(GOLDEN.glob("one_thread_*.npz"))
RECOUNT = sorted(GOLDEN.glob("recount_*.npz"))


def _opt(d, key):
    v = d[key]
    return None if v.size == 0 else v


def test_fixtures_present():
    assert len(ONE_THREAD) == 8 and len(RECOUNT) == 3  # 5 2D and 3 3D one-thread runs


@pytest.mark.parametrize("path", ONE_THREAD, ids=lambda p: p.stem)
def test_restatement_reproduces_reference_run(path):
    d = np.load(path)
    lat = d["lattice_in"].copy()
    area, perim = d["area0"].copy(), d["perim0"].copy()
    fixed = _opt(d, "fixed")
    fixed = None if fixed is None else fixed.astype(bool)
    args = (lat, area, perim, d["J"], list(d["lam_a"]), list(d["tgt_a"]), list(d["lam_p"]),
            list(d["tgt_p"]), float(d["temperature"]), int(d["seed"]), int(d["mcs"]))
    if lat.ndim == 3:  # src/kernels3d.cu, with its neighbour redraw test (:208)
        acc = refmodel.sequential_run_3d(*args, perimeter_on=bool(d["perimeter"]),
                                         stick=_opt(d, "stick"), fixed=fixed)
    else:
        acc = refmodel.sequential_run(*args, perimeter_on=bool(d["perimeter"]),
                                      stick=_opt(d, "stick"), fixed=fixed,
                                      chemo=_opt(d, "chemo"), field=_opt(d, "field"))
    assert acc > 10
    np.testing.assert_array_equal(lat, d["lattice_out"])
    np.testing.assert_array_equal(area, d["area_out"])
    if int(d["perimeter"]):
        np.testing.assert_array_equal(perim, d["perim_out"])


@pytest.mark.parametrize("path", ONE_THREAD + RECOUNT, ids=lambda p: p.stem)
def test_oracle_recount_equals_reference_tables(path):
    d = np.load(path)
    one = "lattice_in" in d.files
    lat = d["lattice_in"] if one else d["lattice"]
    area = d["area0"] if one else d["area"]
    perim = d["perim0"] if one else d["perim"]
    nt = 32
    sim = oracle.OracleSim(lat, int(d["ncells"]), np.zeros((nt, nt), np.float32), [0] * nt,
                           [0] * nt)
    np.testing.assert_array_equal(sim.area, area)
    np.testing.assert_array_equal(sim.perim, perim)
