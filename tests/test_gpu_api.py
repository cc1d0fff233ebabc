"""The reference's Python API on the GPU engine: the three example scripts
(minus their PIL / matplotlib / skimage image code), error behaviour, view
lifetime, and the bounded-barrier failure path."""
import gc
import time

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _run_kw(iterations, tpb=4, ppt=8, ppc=4):
    return dict(cell_sync=0, block_sync=0, global_sync=1, threads_per_block=tpb,
                positions_per_thread=ppt, positions_per_checkerboard=ppc,
                updates_per_checkerboard_switch=1, updates_per_barrier=1,
                iterations=iterations, inner_iterations=iterations)


def _check_tables_against_recount(sim, ncells, ndim):
    area, perim, cs = sim.tables()
    lat = sim.get_state().view(np.uint32)
    J = np.zeros((2, 2), np.float32)
    rec = oracle.OracleSim(lat, ncells, J, [0, 0], [0, 0])
    np.testing.assert_array_equal(area, rec.area)
    np.testing.assert_array_equal(perim, rec.perim)
    n = lat.shape[0]
    assert ((cs - rec.csum) % n == 0).all()


def test_example2d(engine_lib):
    """examples/example2d.py: three cells grow to target area 200."""
    import gpucpm
    dimension = 256
    sim = gpucpm.Cpm(dimension, 2, 10, 20, False)
    sim.add_cell(1, 100, 100)
    sim.add_cell(1, 200, 200)
    sim.add_cell(1, 200, 100)
    sim.set_constraints(cell_type=1, lambda_area=10, target_area=200)
    sim.set_constraints(cell_type=0, other_cell_type=1, adhesion=10)
    sim.push_to_gpu()
    sim.run(**_run_kw(2000))
    sim.synchronize()
    centroids = sim.get_centroids()
    assert centroids.shape == (3, 2)
    assert np.all((centroids >= 0) & (centroids < dimension))
    sim.pull_from_gpu()
    state = sim.get_state()
    ids = state % 2 ** 24
    areas = np.bincount(ids.ravel(), minlength=4)[1:4]
    assert np.all(np.abs(areas - 200) < 40), areas
    _check_tables_against_recount(sim, 10, 2)


def test_example3d(engine_lib):
    """examples/example3d.py: three cells grow to target volume 2000."""
    import gpucpm
    dimension = 64
    sim = gpucpm.Cpm(dimension, 3, 10, 20, False)
    sim.add_cell(1, 16, 16, 16)
    sim.add_cell(1, 48, 48, 32)
    sim.add_cell(1, 32, 16, 48)
    sim.set_constraints(cell_type=1, lambda_area=10, target_area=2000)
    sim.set_constraints(cell_type=0, other_cell_type=1, adhesion=10)
    sim.push_to_gpu()
    sim.run(**_run_kw(300))
    sim.synchronize()
    assert sim.get_centroids().shape == (3, 3)
    sim.pull_from_gpu()
    ids = sim.get_state() % 2 ** 24
    vols = np.bincount(ids.ravel(), minlength=4)[1:4]
    assert np.all(vols > 1000), vols
    _check_tables_against_recount(sim, 10, 3)


def test_sorting_example(engine_lib):
    """examples/sorting.py: state painted through get_state(), then pushed."""
    import gpucpm
    rng = np.random.default_rng(0)
    dimension = 256
    newstate = np.zeros((dimension, dimension), "int32")
    ncells = 1
    for x in range(0, dimension - 1, 6):
        for y in range(0, dimension - 1, 6):
            if (x - dimension / 2) ** 2 + (y - dimension / 2) ** 2 < (dimension ** 2) / 9:
                t = int(rng.integers(1, 3))
                newstate[x:x + 3, y:y + 3] = (t * (2 ** 24)) + ncells
                ncells += 1
    sim = gpucpm.Cpm(dimension, 2, ncells, 10, False)
    sim.set_constraints(cell_type=1, lambda_area=1, target_area=40)
    sim.set_constraints(cell_type=1, other_cell_type=1, adhesion=14)
    sim.set_constraints(cell_type=0, other_cell_type=1, adhesion=16)
    sim.set_constraints(cell_type=2, lambda_area=1, target_area=40)
    sim.set_constraints(cell_type=2, other_cell_type=2, adhesion=2)
    sim.set_constraints(cell_type=2, other_cell_type=1, adhesion=11)
    sim.set_constraints(cell_type=2, other_cell_type=0, adhesion=16)
    state = sim.get_state()
    state[:, :] = newstate
    sim.push_to_gpu()
    sim.run(**_run_kw(1000, tpb=32, ppt=4, ppc=2))
    sim.synchronize()
    sim.pull_from_gpu()
    s = sim.get_state()
    types = s // 2 ** 24
    assert set(np.unique(types)) <= {0, 1, 2}
    _check_tables_against_recount(sim, ncells, 2)


def test_push_rejects_invalid_lattices(engine_lib):
    import gpucpm
    sim = gpucpm.Cpm(32, 2, 4, 10, False)
    st = sim.get_state()
    st[0, 0] = 9 | (1 << 24)  # id above number_of_cells
    with pytest.raises(gpucpm.CpmError, match="above number_of_cells"):
        sim.push_to_gpu()
    st[0, 0] = 1 << 24        # medium carrying a type
    with pytest.raises(gpucpm.CpmError, match="id 0 with a non-zero type"):
        sim.push_to_gpu()
    st[0, 0] = 1 | (1 << 24)
    st[5, 5] = 1 | (2 << 24)  # one id, two types
    with pytest.raises(gpucpm.CpmError, match="two different types"):
        sim.push_to_gpu()
    st[5, 5] = 2 | (40 << 24)  # type beyond the parameter tables
    with pytest.raises(gpucpm.CpmError, match="type >= 32"):
        sim.push_to_gpu()
    with pytest.raises(gpucpm.CpmError, match="before a successful push"):
        sim.run(**_run_kw(5))
    st[5, 5] = 2 | (2 << 24)
    sim.push_to_gpu()
    sim.run(**_run_kw(5))
    sim.synchronize()


def test_optional_terms_and_bad_arguments(engine_lib):
    import gpucpm
    sim = gpucpm.Cpm(32, 2, 4, 10, False)
    # persistence is accepted in 2D and has no effect there, as in the reference
    sim.set_constraints(cell_type=1, lambda_persistence=1.0, persistence_diffusion=0.5,
                        persistence_time=10)
    assert not sim.persistence_exists
    with pytest.raises(gpucpm.CpmError):
        sim.set_history(0)
    # chemotaxis needs the field, which exists (zero) once asked for
    sim.set_constraints(cell_type=1, lambda_chemotaxis=1.0)
    with pytest.raises(gpucpm.CpmError):
        sim.set_constraints(cell_type=40, lambda_area=1, target_area=4)
    with pytest.raises(gpucpm.CpmError):
        sim.add_cell(1, 32, 0)
    with pytest.raises(TypeError):
        sim.run(**{**_run_kw(5), "iterations": 5.5})
    for _ in range(4):
        sim.add_cell(1, 1, 1)
    with pytest.raises(gpucpm.CpmError, match="exceed number_of_cells"):
        sim.add_cell(1, 2, 2)
    assert sim.get_act_state().shape == (32, 32)
    assert sim.get_field().shape == (2, 32, 32)


def test_state_view_keeps_engine_alive(engine_lib):
    import gpucpm
    sim = gpucpm.Cpm(16, 2, 2, 10, False)
    sim.add_cell(1, 3, 3)
    view = sim.get_state()
    del sim
    gc.collect()
    assert view[3, 3] == 1 | (1 << 24)


def test_asymmetric_adhesion_is_honoured(engine_lib):
    import gpucpm
    sim = gpucpm.Cpm(16, 2, 2, 10, False)
    sim.set_constraints(cell_type=1, other_cell_type=2, adhesion=7, set_adhesion_symmetric=0)
    sim.set_constraints(cell_type=2, other_cell_type=1, adhesion=3, set_adhesion_symmetric=0)
    # (no direct getter: parity of asymmetric J is covered by the oracle tests
    # through the C-ABI; here the calls must simply be accepted)


def test_barrier_timeout_is_reported_not_hung(engine_lib):
    import gpucpm
    t0 = time.time()
    status = gpucpm.barrier_timeout_selftest(50_000_000)
    dt = time.time() - t0
    assert status == gpucpm.CPM_ERR_TIMEOUT
    assert dt < 10.0
    # the context is still usable afterwards
    sim = gpucpm.Cpm(16, 2, 2, 10, False)
    sim.add_cell(1, 3, 3)
    sim.push_to_gpu()
    sim.run(**_run_kw(10))
    sim.synchronize()


def test_c_example_matches_python(engine_lib, tmp_path):
    """tests/capi/example2d.c (the C-ABI alone) prints the same centroids as
    the same run through gpucpm.Cpm."""
    import pathlib
    import shutil
    import subprocess

    import gpucpm
    root = pathlib.Path(__file__).resolve().parents[1]
    cc = shutil.which("cc") or shutil.which("gcc")
    assert cc, "no C compiler"
    lib_dir = root / "gpu-cpm_gb300"
    exe = tmp_path / "example2d"
    subprocess.run([cc, "-std=c99", "-I", str(root / "include"),
                    str(root / "tests" / "capi" / "example2d.c"), "-L", str(lib_dir),
                    "-lgpucpm_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    got = np.array([[float(v) for v in line.split()] for line in out.stdout.split("\n") if line])

    sim = gpucpm.Cpm(256, 2, 10, 20, False)
    sim.set_seed(7, 0)
    sim.add_cell(1, 100, 100)
    sim.add_cell(1, 200, 200)
    sim.add_cell(1, 200, 100)
    sim.set_constraints(cell_type=1, lambda_area=10, target_area=200)
    sim.set_constraints(cell_type=0, other_cell_type=1, adhesion=10)
    sim.push_to_gpu()
    sim.run(**_run_kw(2000))
    sim.synchronize()
    want = sim.get_centroids()
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-6)  # printed with 6 decimals


def test_two_engines_interleaved_equal_each_alone(engine_lib):
    """Handles share no state: two engines whose runs interleave on their own
    streams end exactly as each does alone."""
    import gpucpm
    from gpucpm import workloads as W

    def make(w, seed):
        e = gpucpm.create_box(w.lattice.shape[1], w.lattice.shape[0], 1, 2, w.ncells,
                              w.temperature)
        e.lattice(0)[...] = w.lattice.view(np.int32)
        w.apply(e, replica=0)
        e.set_seed(seed, 0)
        e.push_to_gpu()
        return e

    wa = W.random_small((96, 80), 60, seed=31, temperature=9.0)
    wb = W.random_small((64, 72), 40, seed=32, temperature=7.0)
    alone = []
    for w, seed in ((wa, 1), (wb, 2)):
        e = make(w, seed)
        for _ in range(4):
            e.run_mcs(5)
        e.synchronize()
        e.pull_from_gpu()
        alone.append(e.lattice(0).copy())
    ea, eb = make(wa, 1), make(wb, 2)
    for _ in range(4):
        ea.run_mcs(5)
        eb.run_mcs(5)
    for e in (ea, eb):
        e.synchronize()
        e.pull_from_gpu()
    np.testing.assert_array_equal(ea.lattice(0), alone[0])
    np.testing.assert_array_equal(eb.lattice(0), alone[1])


def test_create_run_destroy_does_not_leak(engine_lib):
    """Engines with every optional buffer (field, act stamps, persistence
    state) release all device memory when destroyed."""
    import torch

    import gpucpm

    def cycle():
        sim = gpucpm.Cpm(64, 3, 20, 10, True, 2, 1)
        for k in range(5):
            sim.add_cell(1, 10 + 9 * k, 12, 20)
        sim.set_constraints(cell_type=1, lambda_area=2, target_area=100)
        sim.set_constraints(cell_type=0, other_cell_type=1, adhesion=10)
        sim.set_constraints(cell_type=1, lambda_persistence=5.0, persistence_diffusion=0.5,
                            persistence_time=3)
        sim.push_to_gpu()
        sim.run_mcs(3)
        sim.synchronize()
        assert sim.persistence_exists and sim.act_exists
        del sim
        gc.collect()

    cycle()  # first use: module loads, context growth
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(10):
        cycle()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free0 - free1 < 8 * 1024 * 1024, (free0, free1)  # under one engine's worth
