"""Shared helpers of the parity tests."""
from __future__ import annotations

import numpy as np

from phasta_gb300 import mesh
from phasta_gb300.solver import make_params


def rel(a, b) -> float:
    a, b = np.asarray(a), np.asarray(b)
    d = np.linalg.norm(a - b)
    s = np.linalg.norm(b)
    return float(d / s) if s > 0 else float(d)


def channel(n=8, mach=0.3, sigma=0.01, seed=20261203, ac_scale=0.0, **kw):
    """Channel case (periodic y,z; inflow/outflow in x) with a perturbed state."""
    case, ph = mesh.channel_case(n, mach=mach)
    p = make_params(ph["mu"], ph["dt"], **kw)
    y = mesh.uniform_state(case, mach, sigma=sigma, seed=seed)
    ac = np.zeros_like(y)
    if ac_scale:
        g = np.random.default_rng(seed + 1)
        ac = ac_scale * g.standard_normal(y.shape) * np.repeat(np.abs(y.reshape(5, -1)).mean(axis=1), case.nshg)
        ac = np.ascontiguousarray(ac.reshape(5, -1)[:, case.iper]).reshape(-1)  # slaves carry the masters' values
    return case, p, y, ac


def vortex(n=8, **kw):
    case, ph = mesh.periodic_vortex_case(n)
    p = make_params(ph["mu"], ph["dt"], **kw)
    y = mesh.vortex_state(case)
    return case, p, y, np.zeros_like(y)


def mixed(n_tet=3, n_hex=3, n_wedge=(3, 3, 2), mach=0.3, sigma=0.01, seed=20261203, ac_scale=0.05, **kw):
    """Disjoint periodic tet, hex and wedge blocks with the channel's perturbed free stream."""
    case, ph = mesh.mixed_case(n_tet, n_hex, n_wedge, mach=mach)
    p = make_params(ph["mu"], ph["dt"], **kw)
    y = mesh.uniform_state(case, mach, sigma=sigma, seed=seed)
    ac = np.zeros_like(y)
    if ac_scale:
        g = np.random.default_rng(seed + 1)
        ac = ac_scale * g.standard_normal(y.shape) * np.repeat(np.abs(y.reshape(5, -1)).mean(axis=1), case.nshg)
        ac = np.ascontiguousarray(ac.reshape(5, -1)[:, case.iper]).reshape(-1)
    return case, p, y, ac


def layered(nxy=3, layers=(2, 1, 2), mach=0.3, sigma=0.02, seed=20261203, ac_scale=0.05, periodic_x=True, **kw):
    """One connected box whose hex, prism and tet layers share their interface nodes (periodic, or
    with inflow and outflow faces in x)."""
    case, ph = mesh.layered_case(nxy, *layers, mach=mach, periodic_x=periodic_x)
    p = make_params(ph["mu"], ph["dt"], **kw)
    y = mesh.uniform_state(case, mach, sigma=sigma, seed=seed)
    ac = np.zeros_like(y)
    if ac_scale:
        g = np.random.default_rng(seed + 1)
        ac = ac_scale * g.standard_normal(y.shape) * np.repeat(np.abs(y.reshape(5, -1)).mean(axis=1), case.nshg)
        ac = np.ascontiguousarray(ac.reshape(5, -1)[:, case.iper]).reshape(-1)
    return case, p, y, ac


def _perturbed(case, ph, mach, sigma, seed, ac_scale, **kw):
    p = make_params(ph["mu"], ph["dt"], **kw)
    y = mesh.uniform_state(case, mach, sigma=sigma, seed=seed)
    ac = np.zeros_like(y)
    if ac_scale:
        g = np.random.default_rng(seed + 1)
        ac = ac_scale * g.standard_normal(y.shape) * np.repeat(np.abs(y.reshape(5, -1)).mean(axis=1), case.nshg)
        ac = np.ascontiguousarray(ac.reshape(5, -1)[:, case.iper]).reshape(-1)
    return case, p, y, ac


def hexchannel(n=3, mach=0.3, sigma=0.01, seed=20261203, ac_scale=0.05, **kw):
    """The channel on hexes: inflow and outflow through boundary hexes."""
    case, ph = mesh.channel_hex_case(n, mach=mach)
    return _perturbed(case, ph, mach, sigma, seed, ac_scale, **kw)


def wedgechannel(n=(3, 3, 2), mach=0.3, sigma=0.01, seed=20261203, ac_scale=0.05, **kw):
    """The channel on prisms: quadrilateral inflow/outflow faces, triangle wall faces."""
    case, ph = mesh.channel_wedge_case(n, mach=mach)
    return _perturbed(case, ph, mach, sigma, seed, ac_scale, **kw)
