"""
Tersoff parameter fitting on the GPU.

Energies and forces of a batch of structures are a differentiable function of
the 14 continuous single-element Tersoff parameters

    A, B, lambda, mu, beta, n, c, d, h, R, S, xi, omega, mubo

(tersoff_params.f90 / tersoff_func.f90 naming: R = r1, S = r2, xi = chi) and
of the positions.  ``EnergyForces`` is a ``torch.autograd.Function``: its
forward pass is one batched evaluation, its backward pass one adjoint pass of
the library (gb_batch_tersoff_adjoint): the hand-written reverse-mode
gradient dE_s/dtheta evaluated in dual numbers along v = dL/dF, which gives
in the same pass the parameter gradient of the force term,
d(v . dE/dr)/dtheta, and the Hessian-vector product -H v for the positions
(bond-order intermediates recomputed, nothing stored per triplet).  The
forward-mode tangents (gb_batch_tersoff_tangent, one pass per parameter)
remain available as ``TersoffBatch.evaluate`` and check the adjoint.

No counterpart in the reference (which has no gradients with respect to
parameters); ``fitting_loss`` is the loss of the fitting workload:
mean_s (E_s/N_s - E_t,s/N_s)^2 + w_F mean_i |F_i - F_t,i|^2.
"""

import ctypes

import numpy as np

from . import native
from ._lib import check
from .parameters import Tersoff_PRB_39_5566_Si_C, atomic_numbers, pair_index

try:
    import torch
except Exception:  # pragma: no cover
    torch = None

PARAM_NAMES = ("A", "B", "lambda", "mu", "beta", "n", "c", "d", "h", "R", "S", "xi", "omega",
               "mubo")


def single_element_parameters(params=Tersoff_PRB_39_5566_Si_C, element="Si"):
    """(theta[14], m) of ``element`` from a multi-element parameter dict."""
    els = list(params["el"])
    q = els.index(element)
    t = pair_index(q, q, len(els))
    return np.array([params["A"][t], params["B"][t], params["lambda"][t], params["mu"][t],
                     params["beta"][q], params["n"][q], params["c"][q], params["d"][q],
                     params["h"][q], params["r1"][t], params["r2"][t], params["xi"][t],
                     params["omega"][t], params["mubo"][t]], dtype=np.float64), \
        int(params["m"][t])


def parameter_dict(theta, m=1, element="Si"):
    """Single-element parameter dict (parameters.py format) of theta."""
    th = [float(x) for x in theta]
    return {"el": [element], "A": [th[0]], "B": [th[1]], "lambda": [th[2]], "mu": [th[3]],
            "beta": [th[4]], "n": [th[5]], "c": [th[6]], "d": [th[7]], "h": [th[8]],
            "r1": [th[9]], "r2": [th[10]], "xi": [th[11]], "omega": [th[12]],
            "mubo": [th[13]], "m": [int(m)]}


class TersoffBatch:
    """A batch of structures evaluated with single-element Tersoff parameters
    theta, with directional derivatives."""

    def __init__(self, structures, element="Si", m=1):
        self.batch = native.Batch(structures)
        self.Z = atomic_numbers[element]
        self.m = int(m)
        self.nat = np.array(self.batch.nat, dtype=np.int64)
        self.offsets = self.batch.offsets
        self.sid = np.repeat(np.arange(len(self.nat)), self.nat)
        self._L = self.batch._L

    def set_positions(self, r):
        self.batch.set_positions(r)

    def evaluate(self, theta, dtheta=None, dr=None):
        """(E[nstruct], dE, F (total,3), dF) along (dtheta, dr)."""
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        dt = None if dtheta is None else np.ascontiguousarray(dtheta, dtype=np.float64)
        drv = None if dr is None else np.ascontiguousarray(dr, dtype=np.float64)
        ns, nat = len(self.nat), int(self.offsets[-1])
        e, de = np.zeros(ns), np.zeros(ns)
        f, df = np.zeros((nat, 3)), np.zeros((nat, 3))
        check(self._L.gb_batch_tersoff_tangent(
            self.batch._h, self.Z, self.m, theta.ctypes.data,
            None if dt is None else dt.ctypes.data, None if drv is None else drv.ctypes.data,
            e.ctypes.data, de.ctypes.data, f.ctypes.data, df.ctypes.data), "tersoff_tangent")
        return e, de, f, df

    def adjoint(self, theta, v=None):
        """One adjoint pass: (E[nstruct], F (total,3), Hv (total,3),
        dE/dtheta (nstruct,14), dv_dE/dtheta (nstruct,14)) with Hv the
        derivative of F along v (= -H v) and dv_dE/dtheta the derivative of
        dE_s/dtheta along v (= d(v . dE_s/dr)/dtheta); v = 0 if None."""
        theta = np.ascontiguousarray(theta, dtype=np.float64)
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
        ns, nat = len(self.nat), int(self.offsets[-1])
        e = np.zeros(ns)
        f, hv = np.zeros((nat, 3)), np.zeros((nat, 3))
        g, gd = np.zeros((ns, 14)), np.zeros((ns, 14))
        check(self._L.gb_batch_tersoff_adjoint(
            self.batch._h, self.Z, self.m, theta.ctypes.data,
            None if vv is None else vv.ctypes.data, e.ctypes.data, f.ctypes.data,
            hv.ctypes.data, g.ctypes.data, gd.ctypes.data), "tersoff_adjoint")
        return e, f, hv, g, gd


if torch is not None:
    class EnergyForces(torch.autograd.Function):
        """(E[nstruct], F[total, 3]) = EnergyForces.apply(theta, positions, tb):
        FP64 energies and forces of the TersoffBatch ``tb``; differentiable in
        theta (14) and positions (total, 3)."""

        @staticmethod
        def forward(ctx, theta, positions, tb):
            tb.set_positions(positions.detach().cpu().numpy())
            e, _, f, _ = tb.evaluate(theta.detach().cpu().numpy())
            ctx.tb = tb
            ctx.save_for_backward(theta, positions)
            ctx.f = f
            return (torch.as_tensor(e, dtype=torch.float64, device=theta.device),
                    torch.as_tensor(f, dtype=torch.float64, device=theta.device))

        @staticmethod
        def backward(ctx, gE, gF):
            theta, positions = ctx.saved_tensors
            tb = ctx.tb
            th = theta.detach().cpu().numpy()
            tb.set_positions(positions.detach().cpu().numpy())
            ge = np.zeros(len(tb.nat)) if gE is None else gE.detach().cpu().numpy()
            gf = np.zeros_like(ctx.f) if gF is None else gF.detach().cpu().numpy()
            g_theta = g_pos = None
            if ctx.needs_input_grad[0] or ctx.needs_input_grad[1]:
                # one adjoint pass along v = gF:
                #   dL/dtheta = sum_s gE_s dE_s/dtheta + sum_i gF_i . dF_i/dtheta
                #             = sum_s gE_s dE_s/dtheta - D_v (dE/dtheta)   (F = -dE/dr)
                #   dL/dr_i   = -gE_s(i) F_i + (dF/dr)^T gF,  (dF/dr)^T gF = -H gF = D_v F
                _, f, hv, dedp, dvdedp = tb.adjoint(th, gf)
                if ctx.needs_input_grad[0]:
                    g = ge @ dedp - dvdedp.sum(axis=0)
                    g_theta = torch.as_tensor(g, dtype=theta.dtype, device=theta.device)
                if ctx.needs_input_grad[1]:
                    gp = -ge[tb.sid][:, None] * f + hv
                    g_pos = torch.as_tensor(gp, dtype=positions.dtype, device=positions.device)
            return g_theta, g_pos, None


def sharded_loss_and_gradient(theta, shard, nat, e_target, f_target, w_force=0.1):
    """The fitting loss and its gradients when the structures are sharded
    over ranks (one process per GPU, each holding a contiguous slice of the
    structures, distributed.shard_range) — no counterpart in the reference.

    shard: this rank's structures, with ``evaluate(theta)`` -> (E, dE, F, dF)
    and ``adjoint(theta, v)`` -> (E, F, Hv, dE/dtheta, D_v dE/dtheta) as
    TersoffBatch; nat, e_target, f_target: this rank's atom counts and
    targets.  Collectives (distributed.allreduce_sum; none without a process
    group): one sum over ranks of (sum_s (dE_s/N_s)^2, sum_i |dF_i|^2,
    structures, atoms), which fixes the global means, and one sum of the 14
    parameter-gradient partials.  Returns (loss, dL/dtheta — the same on
    every rank —, dL/dpositions of this rank's atoms)."""
    from . import distributed as D
    theta = np.asarray(theta, dtype=np.float64)
    nat = np.asarray(nat, dtype=np.float64)
    e, _, f, _ = shard.evaluate(theta)
    de = (e - np.asarray(e_target)) / nat
    df = f - np.asarray(f_target)
    tot = D.allreduce_sum([np.sum(de * de), np.sum(df * df), len(de), df.shape[0]])
    loss = tot[0] / tot[2] + w_force * tot[1] / tot[3]
    gE = 2.0 * de / nat / tot[2]          # dL/dE_s
    gF = 2.0 * w_force * df / tot[3]      # dL/dF_i
    _, f, hv, dedp, dvdedp = shard.adjoint(theta, gF)
    g = D.allreduce_sum(gE @ dedp - dvdedp.sum(axis=0))
    sid = np.repeat(np.arange(len(nat)), nat.astype(np.int64))
    g_pos = -gE[sid][:, None] * f + hv
    return float(loss), g, g_pos


def fitting_loss(E, F, nat, E_target, F_target, w_force=0.1):
    """mean_s (E_s/N_s - E_t/N_s)^2 + w_force mean_i |F_i - F_t,i|^2 (torch)."""
    n = torch.as_tensor(np.asarray(nat, dtype=np.float64), device=E.device)
    de = (E - E_target) / n
    df = F - F_target
    return torch.mean(de * de) + w_force * torch.mean(torch.sum(df * df, dim=1))
