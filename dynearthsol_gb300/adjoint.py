"""Reverse mode of the explicit step (des_adjoint_forward/backward).

A window of K steps of the 3D FP64 step, with dt held at the start value,
from a fixed start state, as a function of
* the per-element material fields of des_set_elem_field (capi.EF_*:
  log10 viscosity, shear modulus, cohesion0/1, friction angle0/1, thermal
  conductivity), and
* the prescribed boundary velocities (des_params.vbc_values),
and of the start state itself.  Window.gradients maps the adjoint of the
final state (a seed) to the adjoint of the start state and to the parameter
gradients; Window.run is the forward.  central_fd gives the matching
central finite difference for checking, and WindowFunction wraps the pair
as a torch.autograd.Function (final velocities as the output).
"""
from __future__ import annotations

import numpy as np

from . import capi
from .config import nstr_of
from .solver import DeviceModel

STATE_FIELDS = ("coord", "vel", "temperature", "stress", "plstrain", "volume_old")
DERIVED = ("volume", "mass", "tmass", "volume_n", "shpdx", "shpdy", "shpdz")


class Window:
    """K steps (checkpoint every C) from `start` (a host state dict) on an
    FP64 DeviceModel, with the context's clock (time, dt, steps) at `clock`."""

    def __init__(self, model: DeviceModel, start: dict, clock, nsteps: int, checkpoint_every: int):
        self.m = model
        self.start = {k: v.copy() for k, v in start.items() if k not in DERIVED}
        self.clock = clock
        self.K, self.C = nsteps, checkpoint_every
        wl = model.wl
        self.base_fields = {k: np.asarray(v, dtype=np.float64).copy() for k, v in wl.elem_fields.items()}
        self.base_vbc = np.array([model.cs.params.vbc_values[i] for i in range(capi.NBDRY)])
        self.fields = dict(self.base_fields)
        self.vbc = self.base_vbc.copy()

    # parameters: {capi.EF_*: [nelem]} and/or {'vbc_values': [10]}
    def set_params(self, params: dict | None):
        params = params or {}
        for k, v in params.items():
            if k == "vbc_values":
                self.vbc = np.asarray(v, dtype=np.float64).copy()
                self.m.set_params(vbc_values=self.vbc)
            else:
                self.fields[k] = np.asarray(v, dtype=np.float64).copy()
                self.m.set_elem_field(k, self.fields[k])

    def run(self, params: dict | None = None, state: dict | None = None) -> dict:
        """Forward window; returns the final host state."""
        self.set_params(params)
        st = dict(self.start)
        if state:
            st.update({k: np.ascontiguousarray(v, dtype=np.float64) for k, v in state.items()})
        self.m.upload(st, self.clock)
        self.m.adjoint_forward(self.K, self.C)
        return self.m.download()

    def run_vel(self, params: dict | None = None) -> np.ndarray:
        """Forward window, as run(), returning the final velocities only."""
        self.set_params(params)
        self.m.upload(self.start, self.clock)
        self.m.adjoint_forward(self.K, self.C)
        return self.m.download_fields(("vel",))["vel"]

    def gradients(self, seed: dict):
        """Adjoint of the window last run: (start-state adjoint, parameter gradients)."""
        return self.m.adjoint_backward(seed)

    def chained_gradients(self, seed: dict):
        """The window's adjoint as a chain of K one-step adjoints: the forward
        one step at a time from the start (each end state downloaded), then,
        from the last step back, each step re-run alone and reversed with the
        adjoint of its end state as the seed; the parameter gradients are
        summed over the steps.  This is the K-step adjoint by the chain rule,
        formed without checkpoints or a multi-step tape, so it checks those;
        with each one-step adjoint held to finite differences it checks a
        window over which finite differences themselves fail (over several
        steps with elements on the Mohr-Coulomb yield surface the forward's
        rounding -- stresses near 1e8 Pa returned to the surface, increments
        near 0.1 Pa -- makes the loss rough at any usable step size).
        Returns (final state, start-state adjoint, parameter gradients)."""
        m = self.m
        states, clocks = [], []
        st, clk = dict(self.start), self.clock
        for _ in range(self.K):
            states.append(st)
            clocks.append(clk)
            m.upload(st, clk)
            m.adjoint_forward(1, 1)
            st = {k: v for k, v in m.download().items() if k not in DERIVED}
            clk = m.clock()
        adj, total = seed, None
        for k in reversed(range(self.K)):
            m.upload(states[k], clocks[k])
            m.adjoint_forward(1, 1)
            adj, g = m.adjoint_backward(adj)
            total = g if total is None else {key: total[key] + g[key] for key in g}
        return st, adj, total


def weighted(final: dict, seed: dict) -> float:
    """<seed, final> over the seed's fields: a linear loss whose adjoint is the seed."""
    return float(sum(np.vdot(seed[k], final[k]) for k in seed))


def central_fd(win: Window, seed: dict, dstate: dict | None = None, dparams: dict | None = None,
               params: dict | None = None, h: float = 1.0) -> float:
    """(L(p + h d) - L(p - h d)) / 2h of the linear loss <seed, final state>
    along a direction d in the start state (dstate) and/or the parameters
    (dparams, same keys as Window.set_params); params = the base point."""
    base = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in (params or {}).items()}
    vals = []
    for sgn in (1.0, -1.0):
        p = dict(base)
        for k, d in (dparams or {}).items():
            b = p.get(k)
            if b is None:
                b = win.base_vbc if k == "vbc_values" else win.base_fields.get(k)
                if b is None:
                    raise ValueError(f"no base value for parameter {k}; pass it in params")
            p[k] = b + sgn * h * d
        st = None
        if dstate:
            st = {k: win.start[k] + sgn * h * d for k, d in dstate.items()}
        vals.append(weighted(win.run(p, st), seed))
    win.set_params({**{k: v for k, v in win.base_fields.items()}, "vbc_values": win.base_vbc, **base})
    return (vals[0] - vals[1]) / (2 * h)


def fd5(f, h: float) -> float:
    """Fourth-order central difference f'(0) ~ (-f(2h) + 8 f(h) - 8 f(-h) + f(-2h)) / 12h."""
    return (-f(2 * h) + 8 * f(h) - 8 * f(-h) + f(-2 * h)) / (12 * h)


def adjoint_dot(start_adj: dict, grad: dict, dstate: dict | None = None, dparams: dict | None = None) -> float:
    """The adjoint's directional derivative along the same direction."""
    s = 0.0
    for k, d in (dstate or {}).items():
        s += float(np.vdot(start_adj[k], d))
    for k, d in (dparams or {}).items():
        s += float(np.vdot(grad[k], d))
    return s


def _torch():
    import torch
    return torch


def window_function():
    """torch.autograd.Function over a Window: inputs (log10_visc, shear_modulus,
    cohesion0, cohesion1, friction0, friction1, therm_cond, vbc_values) as
    float64 tensors, output the final velocities [nnode, 3].  A None input
    keeps the window's base value and gets no gradient."""
    torch = _torch()
    order = (capi.EF_LOG10_VISC, capi.EF_SHEAR_MODULUS, capi.EF_COHESION0, capi.EF_COHESION1,
             capi.EF_FRICTION0, capi.EF_FRICTION1, capi.EF_THERM_COND)

    class WindowFunction(torch.autograd.Function):
        @staticmethod
        def forward(ctx, win, *inputs):
            params = {}
            for k, t in zip(order, inputs[:7]):
                if t is not None:
                    params[k] = t.detach().cpu().numpy().astype(np.float64)
            if inputs[7] is not None:
                params["vbc_values"] = inputs[7].detach().cpu().numpy().astype(np.float64)
            final = win.run(params)
            ctx.win = win
            ctx.present = [t is not None for t in inputs]
            return torch.from_numpy(final["vel"].copy())

        @staticmethod
        def backward(ctx, gvel):
            _, grad = ctx.win.gradients({"vel": gvel.detach().cpu().numpy().astype(np.float64)})
            outs = [None]
            for k, pres in zip(order, ctx.present[:7]):
                outs.append(torch.from_numpy(grad[k].copy()) if pres else None)
            outs.append(torch.from_numpy(grad["vbc_values"].copy()) if ctx.present[7] else None)
            return tuple(outs)

    return WindowFunction


def misfit_difference(vel_a: np.ndarray, vel_b: np.ndarray, target: np.ndarray, nodes: np.ndarray) -> float:
    """L(a) - L(b) of the surface-velocity misfit, formed without subtracting
    two nearly equal misfits: 1/2 sum (v_a - v_b)(v_a + v_b - 2 v_target)
    over the nodes (exact algebra; only the velocity differences round)."""
    va, vb, vt = vel_a[nodes], vel_b[nodes], target[nodes]
    return 0.5 * float(np.sum((va - vb) * ((va - vt) + (vb - vt))))


def fd5_misfit(vel_at, h: float, target: np.ndarray, nodes: np.ndarray) -> float:
    """Fourth-order central difference of the misfit along a direction,
    (8 (L(h) - L(-h)) - (L(2h) - L(-2h))) / 12h, each difference taken by
    misfit_difference; vel_at(t) = the final velocities at step t."""
    v = {t: vel_at(t) for t in (h, -h, 2 * h, -2 * h)}
    d1 = misfit_difference(v[h], v[-h], target, nodes)
    d2 = misfit_difference(v[2 * h], v[-2 * h], target, nodes)
    return (8 * d1 - d2) / (12 * h)


def surface_velocity_misfit(final_vel: np.ndarray, target: np.ndarray, nodes: np.ndarray):
    """L = 1/2 sum over the given nodes of |v - v_target|^2 and its seed."""
    r = final_vel[nodes] - target[nodes]
    seed = np.zeros_like(final_vel)
    seed[nodes] = r
    return 0.5 * float(np.sum(r * r)), seed


def state_shapes(model: DeviceModel) -> dict:
    m = model.wl.mesh
    nd, nn, ne = m.ndims, m.nnode, m.nelem
    return {"coord": (nn, nd), "vel": (nn, nd), "temperature": (nn,), "stress": (ne, nstr_of(nd)),
            "plstrain": (ne,), "volume_old": (ne,)}


# --------------------------------------------------------------------------
# the adjoint workload: surface-velocity misfit against a target run
# --------------------------------------------------------------------------
def grf_log10_visc(mesh, mean: float = 21.0, sd: float = 0.5, corr_len: float = 15e3, seed: int = 0,
                   nfeatures: int = 128) -> np.ndarray:
    """Per-element log10 viscosity drawn from a Gaussian random field with a
    squared-exponential covariance sd^2 exp(-r^2 / (2 corr_len^2)), sampled
    at element centroids by random Fourier features (Rahimi and Recht,
    "Random features for large-scale kernel machines", NIPS 2007)."""
    from .config import elem_center
    rng = np.random.default_rng(seed)
    x = elem_center(mesh)
    w = rng.standard_normal((nfeatures, x.shape[1])) / corr_len
    b = rng.uniform(0, 2 * np.pi, nfeatures)
    f = np.sqrt(2.0 / nfeatures) * np.cos(x @ w.T + b).sum(axis=1)
    return mean + sd * f


def top_nodes(mesh) -> np.ndarray:
    """Nodes on the top surface (BOUNDZ1)."""
    from .mesh import BOUNDZ1
    return np.nonzero(mesh.bcflag & BOUNDZ1)[0]


def adjoint_workload(cells=None, seed: int = 12345):
    """The 3D adjoint case on the 998,400-tet box (or `cells`): EVP physics of
    the 3D workload with the continuous damping option 2 and per-element
    fields for every differentiated property.  Returns (workload, target
    log10 viscosity, start log10 viscosity)."""
    from dataclasses import replace
    from .config import make_workload
    wl = make_workload("c1_3d_evp", cells=cells, seed=seed)
    wl.params = replace(wl.params, damping_option=2)
    m, mt = wl.mesh, wl.mat
    ne = m.nelem
    lv_target = grf_log10_visc(m, seed=seed)
    lv_start = grf_log10_visc(m, seed=seed + 1)
    wl.elem_fields = {capi.EF_LOG10_VISC: lv_start,
                      capi.EF_SHEAR_MODULUS: np.full(ne, mt.shear_modulus[0]),
                      capi.EF_COHESION0: np.full(ne, mt.cohesion0[0]),
                      capi.EF_COHESION1: np.full(ne, mt.cohesion1[0]),
                      capi.EF_FRICTION0: np.full(ne, mt.friction_angle0[0]),
                      capi.EF_FRICTION1: np.full(ne, mt.friction_angle1[0])}
    return wl, lv_target, lv_start


def yielding_adjoint_workload(cells=(20, 20, 6), halfwidth: float = 15e3, seed: int = 7):
    """A window in which elements yield: the 3D workload's physics with
    damping option 2 and, as per-element fields, a vertical band of weak
    material (|x - xlength/2| < halfwidth: cohesion 1 -> 0.1 MPa, friction
    10 -> 5 degrees) in which the Mohr-Coulomb return map is active after a
    few hundred steps.  Returns (workload, target cohesion1, start cohesion1):
    the target run perturbs the band's cohesion1 by a seeded +-20 %."""
    from dataclasses import replace
    from .config import elem_center, make_workload
    wl = make_workload("c1_3d_evp", cells=cells, seed=seed)
    wl.params = replace(wl.params, damping_option=2)
    mt = wl.mat
    band = np.abs(elem_center(wl.mesh)[:, 0] - 0.5 * wl.mesh.lengths[0]) < halfwidth
    ne = wl.mesh.nelem
    c0 = np.where(band, 1e6, mt.cohesion0[0])
    c1 = np.where(band, 1e5, mt.cohesion1[0])
    f0 = np.where(band, 10.0, mt.friction_angle0[0])
    f1 = np.where(band, 5.0, mt.friction_angle1[0])
    wl.elem_fields = {capi.EF_SHEAR_MODULUS: np.full(ne, mt.shear_modulus[0]), capi.EF_COHESION0: c0,
                      capi.EF_COHESION1: c1, capi.EF_FRICTION0: f0, capi.EF_FRICTION1: f1}
    rng = np.random.default_rng(seed)
    c1_target = c1 * (1 + 0.2 * rng.uniform(-1, 1, ne) * band)
    return wl, c1_target, c1
