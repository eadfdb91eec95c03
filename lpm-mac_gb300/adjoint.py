"""Adjoint over a load history, with checkpoints every k steps.

The forward pass runs the load steps through ``Lattice.load_step`` and keeps
a device checkpoint (``lpm_checkpoint_save``) before every k-th step.  The
backward pass walks the segments from the last to the first: it restores
the segment's checkpoint, recomputes the segment's steps once while saving
each converged state, then takes the adjoint of each step in reverse order
(``lpm_backward_step`` with accumulate) and frees the segment's states.

Each step's response is F_n = a_n . x + c_n . Pin at its converged state;
the objective J = phi(F_1, ..., F_N) enters through dJ/dF_n.  The gradient
is exact for laws whose state does not evolve with the load (the elastic
law with every bond intact or broken): the converged state of step n then
depends on the parameters only through that step's equilibrium, and the
per-step adjoints add up.  The steps themselves are recomputed exactly as
the forward pass ran them.
"""
import numpy as np

from . import capi


class LoadHistory:
    def __init__(self, lattice, steps, every=1, **step_kwargs):
        """steps: a list of bc lists (``Lattice.load_step`` form), one per
        load step; every: steps per checkpoint segment."""
        self.g = lattice
        self.steps = list(steps)
        self.every = max(int(every), 1)
        self.kw = step_kwargs
        self.checkpoints = {}

    def _step(self, n):
        r = self.g.load_step(self.steps[n], **self.kw)
        if r["status"] != capi.OK:
            raise RuntimeError("load step %d did not converge: %s" % (n, r))
        return r

    def forward(self, seeds):
        """seeds(n) -> (a_n, c_n) (arrays of N*dim or None).  Runs every
        step and returns the responses F_n."""
        self.seeds = seeds
        out = []
        for n in range(len(self.steps)):
            if n % self.every == 0:
                self.checkpoints[n] = self.g.checkpoint_save()
            self._step(n)
            out.append(self.response(n))
        return np.array(out)

    def response(self, n):
        a, c = self.seeds(n)
        J = 0.0
        if a is not None:
            J += float(np.dot(np.asarray(a).ravel(), self.g.download(capi.F_XYZ)[:, :self.g.dim].ravel()))
        if c is not None:
            J += float(np.dot(np.asarray(c).ravel(), self.g.download(capi.F_PIN)[:, :self.g.dim].ravel()))
        return J

    def backward(self, dJdF, cg_tol=1e-12):
        """dJdF: dJ/dF_n for every step.  Returns (dJ/dKn, dJ/dTv) in stored
        bond order and the adjoint CG iterations."""
        first = True
        iters = 0
        nsteps = len(self.steps)
        for s in sorted(self.checkpoints, reverse=True):
            self.g.checkpoint_restore(self.checkpoints[s])
            states = {}
            for n in range(s, min(s + self.every, nsteps)):
                self._step(n)
                states[n] = self.g.checkpoint_save()
            for n in sorted(states, reverse=True):
                self.g.checkpoint_restore(states[n])
                a, c = self.seeds(n)
                w = float(dJdF[n])
                a = None if a is None else w * np.asarray(a, dtype=np.float64)
                c = None if c is None else w * np.asarray(c, dtype=np.float64)
                gk, gt, it, _ = self.g.backward_step(a, c, cg_tol=cg_tol, accumulate=not first)
                first = False
                iters += it
                self.g.checkpoint_drop(states[n])
        return gk, gt, iters

    def close(self):
        for cid in self.checkpoints.values():
            self.g.checkpoint_drop(cid)
        self.checkpoints = {}


def reaction_curve_sensitivity(lattice, steps, group, axis, dparams, tangent_tol=1e-12, **step_kwargs):
    """A load history of the J2 law with its tangent-linear sensitivity
    (``lpm_tangent_begin``): runs the load steps ``steps`` (``load_step``
    bc lists) and returns the reaction curve R_n (the internal force of the
    particles ``group`` along ``axis``, summed, at each step's equilibrium)
    and its derivatives dR_n/dtheta_k along the parameter directions
    ``dparams`` (one row of the law's parameters, or an (N, np) array, per
    direction), shapes (steps,) and (steps, directions).  A response of the
    curve, e.g. sum (R_n - target_n)^2, then has the gradient
    sum 2 (R_n - target_n) dR_n/dtheta.  tangent_tol is the relative residual
    of the tangent solves; step_kwargs go to ``load_step``."""
    g = lattice
    idx = np.asarray(group, dtype=np.int64)
    g.tangent_begin(dparams, tol=tangent_tol)
    R, dR = [], []
    try:
        for n, bcs in enumerate(steps):
            r = g.load_step(bcs, **step_kwargs)
            if r["status"] != capi.OK:
                raise RuntimeError("load step %d did not converge: %s" % (n, r))
            R.append(g.download(capi.F_PIN)[idx, axis].sum())
            dR.append([g.tangent_get(k, capi.T_PIN)[idx, axis].sum() for k in range(len(dparams))])
    finally:
        g.tangent_end()
    return np.array(R), np.array(dR)
