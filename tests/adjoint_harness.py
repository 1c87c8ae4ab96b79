"""Verification harness of the leapfrog adjoint (csg_adjoint_* C-ABI calls).

The two-disk merger of 10,000 stars (no SPH) as a differentiable function of
three orbital parameters — pericentre r_p, inclination of the second disk
(degrees) and relative approach speed v — built in torch around the seeded
disks of csg_generate_ics kinds 5 and 6; a torch.autograd.Function whose
forward and backward are the library's C-ABI forward and adjoint; and the
finite-difference checks (central differences of the frozen-list map, whose
gradient the adjoint computes).

Orbit: the second disk starts 30 scale lengths from the first along +x; the
relative velocity (-v_r, -v_t, 0) has speed v and the tangential part that
gives a Keplerian pericentre r_p for the two total masses; both disks move
about their common centre of mass. The defaults reproduce csg_generate_ics
kind 4 (0.3 v_circ, tangential/radial 0.17, 50 deg).
"""
import math

import numpy as np
import torch

from cosmosim_gb300 import lib
from cosmosim_gb300.abi import BODY_DTYPE

SEP = 30.0


class MergerIC:
    """x0(p), v0(p) for p = (r_p, inclination_deg, v)."""

    def __init__(self, n, seed):
        n1 = n // 2
        self.d1 = lib.generate_ics(5, n1, seed)
        self.d2 = lib.generate_ics(6, n - n1, seed + 1)
        self.m1 = float(self.d1["mass"].sum())
        self.m2 = float(self.d2["mass"].sum())
        self.template = np.concatenate([self.d1, self.d2]).astype(BODY_DTYPE)
        f = lambda b, k: torch.from_numpy(np.stack([b[k + a] for a in "xyz"], 1).copy())
        self.X1, self.V1 = f(self.d1, ""), f(self.d1, "v")
        self.X2, self.V2 = f(self.d2, ""), f(self.d2, "v")

    def base_params(self):
        mt = self.m1 + self.m2
        vrel = 0.3 * math.sqrt(mt / SEP)
        vrad = vrel / math.sqrt(1.0 + 0.17 ** 2)
        L = SEP * 0.17 * vrad
        E = 0.5 * vrel ** 2 - mt / SEP
        r_p = (-mt + math.sqrt(mt * mt + 2.0 * E * L * L)) / (2.0 * E)
        return np.array([r_p, 50.0, vrel])

    def state(self, p):
        """(x0, v0) as (n, 3) float64 tensors, differentiable in p (tensor of 3)."""
        r_p, inc, v = p[0], p[1], p[2]
        mt = self.m1 + self.m2
        E = 0.5 * v * v - mt / SEP
        vt = r_p * torch.sqrt(2.0 * (E + mt / r_p)) / SEP
        vr = torch.sqrt(v * v - vt * vt)
        zero = torch.zeros((), dtype=torch.float64)
        rel_x = torch.stack([zero + SEP, zero, zero])
        rel_v = torch.stack([-vr, -vt, zero])
        t = inc * (math.pi / 180.0)
        c, s = torch.cos(t), torch.sin(t)
        one = zero + 1.0
        R = torch.stack([torch.stack([one, zero, zero]), torch.stack([zero, c, -s]),
                         torch.stack([zero, s, c])])
        x1 = self.X1 - (self.m2 / mt) * rel_x
        v1 = self.V1 - (self.m2 / mt) * rel_v
        x2 = self.X2 @ R.T + (self.m1 / mt) * rel_x
        v2 = self.V2 @ R.T + (self.m1 / mt) * rel_v
        return torch.cat([x1, x2]), torch.cat([v1, v2])

    def bodies(self, x0, v0):
        b = self.template.copy()
        x0 = np.asarray(x0, dtype=np.float64).reshape(-1, 3)
        v0 = np.asarray(v0, dtype=np.float64).reshape(-1, 3)
        for k, a in enumerate("xyz"):
            b[a] = x0[:, k]
            b["v" + a] = v0[:, k]
        return b


class LeapfrogLoss(torch.autograd.Function):
    """loss = mean |x_T - target|^2 of the library's leapfrog run from (x0, v0);
    backward = the library's adjoint."""

    @staticmethod
    def forward(ctx, x0, v0, adj, ic, target, record):
        b = ic.bodies(x0.detach().numpy(), v0.detach().numpy())
        loss = adj.forward(b, target, record=record)
        ctx.adj = adj
        return x0.new_tensor(loss)

    @staticmethod
    def backward(ctx, g):
        gx, gv = ctx.adj.backward()
        return g * torch.from_numpy(gx), g * torch.from_numpy(gv), None, None, None, None


class MergerProblem:
    def __init__(self, n=10000, seed=0xAD70, substeps=200, dt=2e-3, checkpoint_every=20,
                 softening=0.01, theta=0.5, mode=lib.ADJ_TREE, target_shift=(1.05, 2.0, 0.97)):
        self.ic = MergerIC(n, seed)
        self.n = n
        self.p0 = self.ic.base_params()
        self.adj = lib.Adjoint(n, softening=softening, theta=theta, dt=dt, substeps=substeps,
                               checkpoint_every=checkpoint_every, mode=mode)
        # seeded target snapshot: the final positions of the run from nearby
        # orbital parameters
        pt = self.p0 * np.array([target_shift[0], 1.0, target_shift[2]])
        pt[1] += target_shift[1]
        xt, vt = self.ic.state(torch.tensor(pt))
        _, fin = self.adj.forward(self.ic.bodies(xt.numpy(), vt.numpy()), np.zeros((n, 3)),
                                  final=True)
        self.target = np.stack([fin["x"], fin["y"], fin["z"]], 1)

    def gradients(self, record=True):
        """Loss, dL/dp (3), dL/dx0, dL/dv0 through the autograd Function."""
        p = torch.tensor(self.p0, requires_grad=True)
        x0, v0 = self.ic.state(p)
        x0.retain_grad()
        v0.retain_grad()
        loss = LeapfrogLoss.apply(x0, v0, self.adj, self.ic, self.target, record)
        loss.backward()
        self.z0 = (x0.detach().numpy().copy(), v0.detach().numpy().copy())
        return (loss.item(), p.grad.numpy().copy(), x0.grad.numpy().copy(),
                v0.grad.numpy().copy())

    def frozen_loss(self, x0, v0):
        return self.adj.forward_frozen(self.ic.bodies(x0, v0), self.target)

    def fd_directions(self, gx, gv, k=32, h=1e-6, seed=7, frozen=True):
        """Central differences along k random unit directions of (x0, v0) space
        against the adjoint's directional derivative."""
        rng = np.random.default_rng(seed)
        x0, v0 = self.z0
        out = []
        for _ in range(k):
            u = rng.standard_normal(6 * self.n)
            u /= np.linalg.norm(u)
            ux, uv = u[:3 * self.n].reshape(-1, 3), u[3 * self.n:].reshape(-1, 3)
            if frozen:
                lp = self.frozen_loss(x0 + h * ux, v0 + h * uv)
                lm = self.frozen_loss(x0 - h * ux, v0 - h * uv)
            else:
                lp = self.adj.forward(self.ic.bodies(x0 + h * ux, v0 + h * uv), self.target)
                lm = self.adj.forward(self.ic.bodies(x0 - h * ux, v0 - h * uv), self.target)
            fd = (lp - lm) / (2 * h)
            ad = float((gx * ux).sum() + (gv * uv).sum())
            out.append((fd, ad))
        return out

    def fd_params(self, gp, h=1e-6):
        """Central differences in each orbital parameter (frozen lists)."""
        out = []
        for k in range(3):
            e = np.zeros(3)
            e[k] = h
            lp = self.frozen_loss(*[t.numpy() for t in self.ic.state(torch.tensor(self.p0 + e))])
            lm = self.frozen_loss(*[t.numpy() for t in self.ic.state(torch.tensor(self.p0 - e))])
            out.append(((lp - lm) / (2 * h), float(gp[k])))
        return out

    def close(self):
        self.adj.close()


def rel_errors(pairs):
    return [abs(fd - ad) / max(abs(ad), 1e-300) for fd, ad in pairs]


def floored_errors(pairs, gnorm, floor=1e-3):
    """|fd - ad| / max(|ad|, floor |grad|): the relative error, except for
    directions almost orthogonal to the gradient, where the difference
    quotient's own rounding (loss rounding / h) dominates |ad|."""
    return [abs(fd - ad) / max(abs(ad), floor * gnorm, 1e-300) for fd, ad in pairs]
