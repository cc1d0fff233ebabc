"""Likelihood-ratio gradients of ensemble observables, as a torch.autograd op.

An `Ensemble` holds R independent 2D replicas (one gpucpm.Batch) that share
the parameter vector

    theta = (J of each listed type pair..., lambda_area, [lambda_perim,] T)

J pairs are symmetric adhesions; lambda_area (lambda_perim) is one value set
on every cell type 1.. of the workloads, each type keeping its own area
(perimeter) target; T is the temperature.  Every
forward pass restarts all replicas from their initial lattices and Monte
Carlo time 0, runs the sweep with the engine's score accumulation (the
forward kernel sums d log P(decision)/d theta of every attempt, per replica
and MCS, in FP32) and measures the sorting order parameter O at the
requested checkpoints.  `LikelihoodRatio.apply(theta, ens, mcs, checkpoints)`
returns O as a [R, C] tensor; its backward runs the engine's backward
kernel

    dE[L]/dtheta_k ~ sum_r sum_c dL/dO[r,c] (O[r,c] - b[r,c])
                                  * sum_{t < checkpoint_c} score[r,t,k]

(score-function estimator; b[r,c] is the mean of O[.,c] over the other
replicas, which keeps it unbiased).  For L = mean_r f(O[r]) this estimates
d E[f(O)] / d theta.
Because the Philox stream is a pure function of (seed, replica, site,
phase), two forward passes with the same seed use common random numbers,
which is what `crn_finite_difference` relies on.

Sharded ensembles: with `group` (a torch.distributed process group, one
process per GPU, each holding its own replicas with distinct stream ids),
backward all-reduces the per-checkpoint sums of O and the replica count
before the backward kernel, so that the baseline runs over every shard's
replicas, and all-reduces the gradient after it (averaged over shards, the
convention of data-parallel training: each shard's loss is the mean over
its own replicas).  These two small all-reduces are the only collectives.
"""
import numpy as np
import torch

import gpucpm


class Ensemble:
    def __init__(self, workloads, pairs=((1, 1), (2, 2), (1, 2), (1, 0), (2, 0)),
                 lambda_area=True, temperature=True, seed=0, stream_id=0, device=0,
                 lambda_perim=False, group=None):
        if any(w.ndim != 2 for w in workloads):
            raise ValueError("likelihood-ratio ensembles are 2D")
        self.workloads = list(workloads)
        self.group = group
        self.spec = gpucpm.ScoreSpec.make(pairs, lambda_area, temperature, lambda_perim)
        self.pairs = [tuple(p) for p in pairs]
        self.seed, self.stream_id = int(seed), int(stream_id)
        self.device = torch.device("cuda", device)
        self.batch = gpucpm.Batch(2, [w.lattice.shape[::-1] for w in self.workloads],
                                  [w.ncells for w in self.workloads])
        self.stream = torch.cuda.Stream(device=self.device)
        self.batch.set_stream(self.stream.cuda_stream)
        self.batch.set_seed(self.seed, self.stream_id)
        # replicas built from one Workload object share its parameters, which
        # are then set once for all replicas (replica None)
        self._shared = all(w is self.workloads[0] for w in self.workloads)
        if self._shared:
            w = self.workloads[0]
            nt = w.J.shape[0]
            for a in range(nt):
                for b in range(nt):
                    self.batch.set_adhesion(None, a, b, float(w.J[a, b]), symmetric=False)
                self.batch.set_area(None, a, int(w.tgt_area[a]), float(w.lam_area[a]))
                self.batch.set_perimeter(None, a, int(w.tgt_perim[a]), float(w.lam_perim[a]))
            self.batch.set_temperature(None, w.temperature)
        else:
            for r, w in enumerate(self.workloads):
                w.apply(self.batch, replica=r)
        self.cell_types = sorted({t for w in self.workloads for t in range(1, w.J.shape[0])})
        self._views = [self.batch.lattice(r) for r in range(len(self.workloads))]
        self._initial = {id(w): w.lattice.view(np.int32) for w in self.workloads}

    @property
    def nparam(self):
        return self.spec.nparam

    def theta0(self):
        """theta of the first workload (J pairs, its lambdas of type 1, its T)."""
        w = self.workloads[0]
        vals = [float(w.J[a, b]) for a, b in self.pairs]
        if self.spec.lambda_area:
            vals.append(float(w.lam_area[self.cell_types[0]]))
        if self.spec.lambda_perim:
            vals.append(float(w.lam_perim[self.cell_types[0]]))
        if self.spec.temperature:
            vals.append(float(w.temperature))
        return torch.tensor(vals, dtype=torch.float64)

    def _apply_theta(self, theta):
        th = [float(v) for v in theta]
        k = 0
        for a, b in self.pairs:  # the same value on every replica
            self.batch.set_adhesion(None, a, b, th[k], symmetric=True)
            k += 1
        # lambdas keep each replica's own targets
        reps = [(None, self.workloads[0])] if self._shared else list(enumerate(self.workloads))
        if self.spec.lambda_area:
            for r, w in reps:
                for t in self.cell_types:
                    self.batch.set_area(r, t, int(w.tgt_area[t]), th[k])
            k += 1
        if self.spec.lambda_perim:
            for r, w in reps:
                for t in self.cell_types:
                    self.batch.set_perimeter(r, t, int(w.tgt_perim[t]), th[k])
            k += 1
        if self.spec.temperature:
            self.batch.set_temperature(None, th[k])

    def _restart(self):
        for v, w in zip(self._views, self.workloads):
            v[...] = self._initial[id(w)]
        self.batch.push_to_gpu()
        self.batch.tick = 0
        self.batch.reset_counters()

    def forward(self, theta, mcs, checkpoints=None, scores=True):
        """Run all replicas from their initial state for `mcs` MCS.

        Returns (O [R, C] float32 cuda tensor, scores [R, mcs, 8] float32
        cuda tensor or None).  checkpoints: MCS counts at which O is
        measured (default: [mcs])."""
        checkpoints = sorted(set(int(c) for c in (checkpoints or [mcs])))
        if checkpoints[-1] > mcs or checkpoints[0] < 1:
            raise ValueError("checkpoints must lie in [1, mcs]")
        self._apply_theta(theta)
        self._restart()
        R = len(self.workloads)
        sc = (torch.zeros((R, mcs, gpucpm.SCORE_MAX), dtype=torch.float32, device=self.device)
              if scores else None)
        obs = []
        done = 0
        torch.cuda.current_stream(self.device).synchronize()
        for c in checkpoints:
            if c > done:
                if scores:
                    self.batch.run_scores(c - done, sc.data_ptr(), 0, mcs, self.spec)
                else:
                    self.batch.run_mcs(c - done)
                done = c
            self.batch.synchronize()
            obs.append(self.batch.observe_heterotypic())
        O = torch.tensor(np.stack(obs, axis=1), dtype=torch.float32, device=self.device)
        return O, sc, checkpoints


class LikelihoodRatio(torch.autograd.Function):
    """O = LikelihoodRatio.apply(theta, ensemble, mcs, checkpoints)."""

    @staticmethod
    def forward(ctx, theta, ensemble, mcs, checkpoints=None):
        O, sc, cps = ensemble.forward(theta.detach().cpu(), int(mcs), checkpoints, True)
        ctx.ensemble, ctx.cps, ctx.mcs = ensemble, cps, int(mcs)
        ctx.theta_dtype, ctx.theta_device = theta.dtype, theta.device
        ctx.save_for_backward(O, sc)
        return O

    @staticmethod
    def backward(ctx, grad_O):
        O, sc = ctx.saved_tensors
        ens = ctx.ensemble
        dl = grad_O.detach().to(device=O.device, dtype=torch.float32).contiguous()
        grad = torch.zeros(ens.nparam, dtype=torch.float32, device=O.device)
        stream = torch.cuda.current_stream(O.device)
        tot, ntot = (None, 0) if ens.group is None else shard_totals(O, ens.group)
        gpucpm.lr_backward(sc.data_ptr(), dl.data_ptr(), O.contiguous().data_ptr(), ctx.cps,
                           O.shape[0], ctx.mcs, ens.nparam, grad.data_ptr(),
                           stream.cuda_stream, obs_total=tot, nrep_total=ntot)
        if ens.group is not None:
            reduce_gradient(grad, ens.group)
        return grad.to(ctx.theta_device, ctx.theta_dtype), None, None, None


def shard_totals(O, group=None):
    """Sum of O[:, c] over the replicas of every shard (one float per
    checkpoint) and the number of those replicas: one all-reduce."""
    import torch.distributed as dist
    buf = torch.cat([O.detach().double().sum(dim=0),
                     torch.tensor([float(O.shape[0])], dtype=torch.float64, device=O.device)])
    dist.all_reduce(buf, group=group)
    vals = buf.cpu().tolist()
    return vals[:-1], int(round(vals[-1]))


def reduce_gradient(grad, group=None):
    """Average of the shards' gradients, in place: one all-reduce."""
    import torch.distributed as dist
    dist.all_reduce(grad, group=group)
    grad /= dist.get_world_size(group)
    return grad


def crn_finite_difference(ensemble, theta, mcs, rel_step=0.01, checkpoint=None,
                          per_replica=False, params=None):
    """Central differences of mean_r O at `checkpoint` (default: mcs) with
    step rel_step * |theta_k| (rel_step for a zero entry), every pair of runs
    on the same random numbers.  With per_replica, also returns the [R, K]
    per-replica differences whose mean over replicas is the estimate.
    `params` (indices) limits the differences to those parameters; the
    others are NaN."""
    theta = torch.as_tensor(theta, dtype=torch.float64)
    cp = [checkpoint or mcs]
    cols = []
    R = len(ensemble.workloads)
    for k in range(len(theta)):
        if params is not None and k not in params:
            cols.append(torch.full((R,), float("nan"), dtype=torch.float64))
            continue
        h = rel_step * (abs(float(theta[k])) or 1.0)
        tp, tm = theta.clone(), theta.clone()
        tp[k] += h
        tm[k] -= h
        op = ensemble.forward(tp, mcs, cp, scores=False)[0][:, 0].double()
        om = ensemble.forward(tm, mcs, cp, scores=False)[0][:, 0].double()
        cols.append(((op - om) / (2 * h)).cpu())
    d = torch.stack(cols, dim=1)
    return (d.mean(dim=0), d) if per_replica else d.mean(dim=0)
