"""Generate the golden fixtures of tests/golden/ from the reference's own
CUDA build (needs a GPU and oracle/_ref, i.e. run where the reference
checkout was built; writes one .npz per case into --out).

Two kinds of fixture:

  one_thread_*.npz  a one-thread run of the reference's sweep
                    (src/kernels2d.cu:44-583, one_thread_3d_*:
                    src/kernels3d.cu:51-594, with threads_per_block = 1 and
                    positions_per_thread = positions_per_checkerboard = D,
                    deterministic for a seed): the input lattice and
                    parameters, the reference's recounted tables before the
                    run, and its lattice and tables after `mcs` MCS.
  recount_*.npz     a lattice and the reference's
                    calculateAreasAndCircumferences tables of it
                    (src/kernels2d.cu:5-41, src/kernels3d.cu:3-47).

tests/test_golden_reference.py checks tests/refmodel.py and the oracle
against these files on the CPU.

    python tests/golden/make_reference_golden.py --out tests/golden
"""
import argparse
import pathlib
import sys

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
for p in (ROOT, ROOT / "gpu-cpm_gb300", ROOT / "tests"):
    sys.path.insert(0, str(p))

from gpucpm import workloads as W  # noqa: E402
from oracle import ref_gpu  # noqa: E402

ONE_THREAD = [  # (D, perimeter, seed, extra terms)
    (16, False, 12345, None),
    (16, True, 777, None),
    (32, True, 31337, None),
    (32, True, 4242, "fixed_sticky"),
    (32, False, 2024, "chemotaxis"),
]
MCS = 3
ONE_THREAD_3D = [  # (D, perimeter, seed, extra terms); D a power of two
    (8, False, 999, None),
    (16, True, 555, None),
    (16, True, 8080, "fixed_sticky"),
]
MCS_3D = 2


def one_thread_case(D, perimeter, seed, terms):
    nt = 3 if terms == "fixed_sticky" else 2
    w = W.random_small((D, D), D * D // 20, ntypes=nt, seed=D + seed % 97, temperature=6.0,
                       perim=perimeter)
    J = np.rint(w.J).astype(np.int64)
    lam_a = np.array([0.0] + [1.0] * nt)
    tgt_a = np.array([0] + [20] * nt)
    lam_p = np.array(([0.0] + [0.5] * nt) if perimeter else [0.0] * (nt + 1))
    tgt_p = np.array([0] + [18] * nt)
    stick = fixed = chemo = field = None
    if terms == "fixed_sticky":
        stick = np.zeros((nt + 1, nt + 1), np.float32)
        stick[1, 2], stick[2, 1], stick[1, 0], stick[0, 2] = 3, 2, 4, 1
        fixed = np.array([False, False, False, True])
    if terms == "chemotaxis":
        chemo = np.array([0.0, 3.0, -2.0], np.float32)
        field = np.random.default_rng(seed).uniform(-2.0, 2.0, (2, D, D))
    wi = W.Workload("one_thread", w.lattice, w.ncells, J.astype(np.float32),
                    lam_a.astype(np.float32), tgt_a.astype(np.int32),
                    lam_p.astype(np.float32), tgt_p.astype(np.int32), 6.0, 0,
                    stick=stick, fixed=fixed, chemo=chemo, field=field)
    return wi, dict(J=J, lam_a=lam_a, tgt_a=tgt_a, lam_p=lam_p, tgt_p=tgt_p)


def one_thread_case_3d(D, perimeter, seed, terms):
    nt = 3 if terms == "fixed_sticky" else 2
    w = W.random_small((D, D, D), D ** 3 // 40, ntypes=nt, seed=D + seed % 89,
                       temperature=6.0, perim=perimeter)
    J = np.rint(w.J).astype(np.int64)
    lam_a = np.array([0.0] + [1.0] * nt)
    tgt_a = np.array([0] + [40] * nt)
    lam_p = np.array(([0.0] + [0.5] * nt) if perimeter else [0.0] * (nt + 1))
    tgt_p = np.array([0] + [90] * nt)
    stick = fixed = None
    if terms == "fixed_sticky":
        stick = np.zeros((nt + 1, nt + 1), np.float32)
        stick[1, 2], stick[2, 1], stick[1, 0], stick[0, 2] = 3, 2, 4, 1
        fixed = np.array([False, False, False, True])
    wi = W.Workload("one_thread_3d", w.lattice, w.ncells, J.astype(np.float32),
                    lam_a.astype(np.float32), tgt_a.astype(np.int32),
                    lam_p.astype(np.float32), tgt_p.astype(np.int32), 6.0, 0,
                    stick=stick, fixed=fixed)
    return wi, dict(J=J, lam_a=lam_a, tgt_a=tgt_a, lam_p=lam_p, tgt_p=tgt_p)


def run_one_thread(out, name, wi, prm, D, ndim, seed, mcs, perimeter):
    ref = ref_gpu.RefGpu(D, ndim, wi.ncells, wi.temperature)
    ref.apply(wi)
    ref.push(wi.lattice)
    area0, perim0 = ref.tables()
    ref.run(mcs, threads_per_block=1, positions_per_thread=D, positions_per_checkerboard=D,
            seed=seed)
    ref.synchronize()
    lat_out = ref.pull()
    area1, perim1 = ref.tables()
    empty = np.zeros(0)
    np.savez_compressed(
        out / f"{name}.npz", lattice_in=wi.lattice.astype(np.uint32), ncells=wi.ncells,
        temperature=6.0, seed=seed, mcs=mcs, perimeter=int(perimeter), **prm,
        stick=empty if wi.stick is None else wi.stick,
        fixed=empty if wi.fixed is None else wi.fixed.astype(np.int32),
        chemo=empty if wi.chemo is None else wi.chemo,
        field=empty if wi.field is None else wi.field,
        area0=area0.astype(np.int64), perim0=perim0.astype(np.int64),
        lattice_out=lat_out.astype(np.uint32), area_out=area1.astype(np.int64),
        perim_out=perim1.astype(np.int64))
    print("wrote", name)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(ROOT / "tests" / "golden"))
    out = pathlib.Path(ap.parse_args().out)
    out.mkdir(parents=True, exist_ok=True)
    if not ref_gpu.available():
        sys.exit("the reference cubin (oracle/_ref) is not built")

    for D, perimeter, seed, terms in ONE_THREAD:
        wi, prm = one_thread_case(D, perimeter, seed, terms)
        name = f"one_thread_D{D}_{'perim' if perimeter else 'noperim'}_{seed}_{terms or 'plain'}"
        run_one_thread(out, name, wi, prm, D, 2, seed, MCS, perimeter)
    for D, perimeter, seed, terms in ONE_THREAD_3D:
        wi, prm = one_thread_case_3d(D, perimeter, seed, terms)
        name = (f"one_thread_3d_D{D}_{'perim' if perimeter else 'noperim'}_{seed}_"
                f"{terms or 'plain'}")
        run_one_thread(out, name, wi, prm, D, 3, seed, MCS_3D, perimeter)

    for name, w in (("recount_sorting64", W.sorting_2d(n=64, ncells=60, seed=3)),
                    ("recount_tissue128", W.tissue_2d(n=128, area=100, seed=4)),
                    ("recount_tissue3d32", W.tissue_3d(n=32, volume=500, seed=5))):
        ref = ref_gpu.RefGpu(w.lattice.shape[0], w.ndim, w.ncells, w.temperature)
        ref.apply(w)
        ref.push(w.lattice)
        area, perim = ref.tables()
        np.savez_compressed(out / f"{name}.npz", lattice=w.lattice.astype(np.uint32),
                            ncells=w.ncells, area=area.astype(np.int64),
                            perim=perim.astype(np.int64))
        print("wrote", name)


if __name__ == "__main__":
    main()
