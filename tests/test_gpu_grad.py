"""Likelihood-ratio scores, the order-parameter kernel, the backward kernel
and the torch.autograd wrapper.

* The forward kernel's FP32 scores (per replica and MCS) equal the oracle's
  FP64 scores computed from the same decisions, within FP32 summation
  error; scoring does not change the dynamics (bit-identical lattices).
* The order-parameter kernel equals a NumPy count on the pulled lattices.
* The backward kernel equals the estimator evaluated in NumPy from the
  same scores, observables and dL/dO; the autograd op returns it as
  theta.grad.
"""
import numpy as np
import pytest

import oracle
import refmodel
from gpucpm import workloads as W

pytestmark = pytest.mark.gpu

PAIRS = ((1, 1), (2, 2), (1, 2), (1, 0), (2, 0))


def _ensemble_workloads(n=3, side=48, seed=50):
    out = []
    for r in range(n):
        w = W.sorting_2d(n=side + 8 * r, ncells=40 + 10 * r, seed=seed + r)
        out.append(w)
    return out


@pytest.mark.parametrize("variant", [None, 3])
def test_scores_match_oracle_and_leave_dynamics_unchanged(engine_lib, variant):
    """variant None: the engine's default tile; 3: the one-row tile, whose
    score kernels have their own instantiation."""
    import torch

    import gpucpm
    ws = _ensemble_workloads()
    spec = gpucpm.ScoreSpec.make(PAIRS, lambda_perim=True)
    b = gpucpm.Batch(2, [w.lattice.shape[::-1] for w in ws], [w.ncells for w in ws])
    if variant is not None:
        b.set_variant(variant)
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.set_seed(21, 5)
    b.push_to_gpu()
    mcs = 12
    sc = torch.zeros((len(ws), mcs, gpucpm.SCORE_MAX), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    b.run_scores(mcs, sc.data_ptr(), 0, mcs, spec)
    b.synchronize()
    b.pull_from_gpu()
    got = sc.cpu().numpy()
    ospec = oracle.ScoreSpec.make(PAIRS, lambda_perim=True)
    for r, w in enumerate(ws):
        sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=21, stream=5 + r)
        want = sim.run_scores(mcs, ospec)
        np.testing.assert_array_equal(b.lattice(r).view(np.uint32), sim.lattice)
        # FP32 per-attempt terms and FP32 sums against FP64: relative to the
        # largest |score| of the parameter over the run
        scale = np.abs(want).max(axis=0) + 1e-6
        err = np.abs(got[r] - want) / scale
        assert err.max() < 2e-3, (r, err.max(axis=0))
        assert (np.abs(want).sum(axis=0) > 0).all()


def test_order_parameter_kernel(engine_lib):
    import gpucpm
    ws = _ensemble_workloads()
    b = gpucpm.Batch(2, [w.lattice.shape[::-1] for w in ws], [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.push_to_gpu()
    b.run_mcs(20)
    b.synchronize()
    b.pull_from_gpu()
    got = b.observe_heterotypic()
    for r in range(len(ws)):
        want = refmodel.heterotypic_fraction(b.lattice(r).view(np.uint32))
        assert abs(float(got[r]) - want) < 1e-6


def test_backward_kernel_and_autograd(engine_lib):
    import torch

    from gpucpm import grad as G
    ws = _ensemble_workloads(n=4)
    ens = G.Ensemble(ws, pairs=PAIRS, seed=3)
    theta = ens.theta0().clone().requires_grad_(True)
    mcs, cps = 16, [8, 16]
    O = G.LikelihoodRatio.apply(theta, ens, mcs, cps)
    assert O.shape == (4, 2)
    w_c = torch.tensor([0.3, 1.0], device=O.device)
    loss = (O * w_c).sum() / O.shape[0]
    loss.backward()
    # the same estimator in NumPy from the same forward
    O2, sc, cps2 = ens.forward(theta.detach(), mcs, cps, scores=True)
    np.testing.assert_array_equal(O.detach().cpu().numpy(), O2.cpu().numpy())
    o = O2.cpu().numpy().astype(np.float64)
    dl = np.tile(w_c.cpu().numpy() / 4.0, (4, 1))
    want, scale = _estimator(sc.cpu().numpy().astype(np.float64), o, dl, cps2, ens.nparam)
    got = theta.grad.numpy()
    # FP32 sums of mixed-sign terms: error bounded relative to sum |term|
    assert (np.abs(got - want) <= 1e-4 * scale).all(), (got, want, scale)
    # the CPU reference gradient: oracle FP64 scores of the same decisions
    ospec = oracle.ScoreSpec.make(PAIRS)
    s_or = np.stack([oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=3,
                                      stream=r).run_scores(mcs, ospec)
                     for r, w in enumerate(ws)])
    ref, scale = _estimator(s_or, o, dl, cps2, ens.nparam)
    assert (np.abs(got - ref) <= 2e-3 * scale).all(), (got, ref, scale)


def _estimator(s, o, dl, cps, nparam):
    """sum_r sum_c dl[r,c] (o[r,c] - leave-one-out mean) * cumulative score,
    and the sum of the absolute values of its terms."""
    R = o.shape[0]
    want = np.zeros(nparam)
    scale = np.zeros(nparam)
    for c, t in enumerate(cps):
        cum = s[:, :t, :nparam].sum(axis=1)
        b = (o[:, c].sum() - o[:, c]) / (R - 1)
        term = (dl[:, c] * (o[:, c] - b))[:, None] * cum
        want += term.sum(axis=0)
        scale += np.abs(term).sum(axis=0)
    return want, scale
