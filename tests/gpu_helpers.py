"""Per-step, per-pass parity of the GPU step against the FP64 oracle, from a shared state.

Each pass is checked on the inputs it consumed:
  density pass            vs the oracle's density pass on the same FP32 positions
  force + integrate pass  vs the oracle's force/integrate passes on the same FP32 state and the
                          densities/pressures the GPU density pass produced
(checking the force against oracle densities instead would mix in the FP32 density rounding,
~2e-7 relative, amplified by the EOS stiffness k wherever rho is near rho0).

Tolerances:
  density   |rho_gpu - rho_ref| / rho_ref                  <= 1e-5  (compensated FP32 sum)
  pressure  |p_gpu - p_ref| / (k * rho_ref)                 <= 1e-5  (p = k (rho - rho0))
  force     |F_gpu - F_ref| <= 1e-5 * S_i + C_R * K_i
            S_i = sum_j |f_ij| + rho_i |G|    (scale: pressure terms cancel inside the fluid)
            K_i = sum_j |f_ij(p)| 2r/(h-r) + |f_ij(v)| r/(h-r)   (conditioning, oracle fcond)
            C_R = 16 * 2^-24: a relative rounding of the pair distance r of 16 FP32 ulps.
            The spiky term (h-r)^2 (force_comp.glsl:59) makes a pair at r -> h ill-conditioned:
            the reference's own FP32 arithmetic on the same inputs misses the plain 1e-5 * S_i
            bound (8e-5 on a 10k-particle gas state; test_oracle_pins checks it meets this one).
  velocity  |v_gpu - v_ref|_inf <= 1e-5 |v|_inf + dt * (force bound) / rho
  position  |x_gpu - x_ref|_inf <= 2e-6 (1 + |x|_inf) + dt * (velocity bound)
Wall clamp (integrate_comp.glsl:45-77): where the unclamped new position lies within
2e-6 (1 + |x|) of a wall plane, FP32 and FP64 may disagree on whether the clamp fires.
Such particles are checked per axis against both outcomes: velocity v_pre or
-damping * v_pre (v_pre = v + dt F / rho), position x_pre or the wall.
"""
from __future__ import annotations

import numpy as np

TOL = 1e-5
C_R = 16.0 * 2.0 ** -24


def force_bound(o: dict, tol: float = TOL) -> np.ndarray:
    return tol * o["fscale"] + C_R * o["fcond"]


def check_step(orc, params, before: np.ndarray, after: np.ndarray, check_force: bool = True, tol: float = TOL,
               backend: str = "grid") -> dict:
    od = orc.step_f64(params, before, backend=backend)
    rho = od["rho"]
    err = {}
    g_rho = after["extras"][:, 0].astype(np.float64)
    g_pres = after["extras"][:, 1].astype(np.float64)
    err["rho"] = float(np.max(np.abs(g_rho - rho) / rho))
    err["pres"] = float(np.max(np.abs(g_pres - od["pres"]) / (params.gas_const * rho + 1e-30)))
    # force and integrate from the GPU's own densities
    o = orc.force_f64(params, before, g_rho, g_pres, backend=backend)
    fb = force_bound(o, tol)
    if check_force:
        df = np.linalg.norm(after["force"][:, :3] - o["force"], axis=1)
        err["force_scaled"] = float(np.max(df / o["fscale"]))  # informational
        err["force"] = float(np.max(df / fb)) * tol            # <= tol  <=>  within the bound
    x_in = before["pos"][:, :3].astype(np.float64)
    v_in = before["vel"][:, :3].astype(np.float64)
    v_pre = v_in + params.dt * o["force"] / g_rho[:, None]
    x_pre = x_in + params.dt * v_pre
    amb = o["margin"] <= 2e-6 * (1.0 + np.abs(x_pre).max(axis=1))
    vb = tol * np.abs(v_in).max(axis=1) + params.dt * fb / g_rho
    xb = 2e-6 * (1.0 + np.abs(o["pos"]).max(axis=1)) + params.dt * vb
    gv = after["vel"][:, :3].astype(np.float64)
    gx = after["pos"][:, :3].astype(np.float64)
    ok = ~amb
    verr = np.abs(gv - o["vel"]).max(axis=1) / vb
    err["vel"] = float(np.max(verr[ok])) * tol if ok.any() else 0.0
    perr = np.abs(gx - o["pos"]).max(axis=1) / xb
    err["pos"] = float(np.max(perr[ok])) if ok.any() else 0.0
    # two-outcome check where the clamp is ambiguous
    if amb.any():
        lo = np.array(params.lower[:3])
        hi = np.array(params.upper[:3])
        vs = vb[amb, None]
        xs = xb[amb, None] + 2e-6 * (1.0 + np.abs(x_pre[amb]))
        v_ok = (np.abs(gv[amb] - v_pre[amb]) <= vs) | (np.abs(gv[amb] + params.damping * v_pre[amb]) <= vs)
        x_ok = (np.abs(gx[amb] - x_pre[amb]) <= xs) | (np.abs(gx[amb] - lo) <= xs) | (np.abs(gx[amb] - hi) <= xs)
        assert v_ok.all() and x_ok.all(), ("wall", np.argwhere(~(v_ok & x_ok)))
    err["wall_ambiguous"] = int(amb.sum())
    for k in ("rho", "pres", "force", "vel"):
        if k in err:
            assert err[k] <= tol, (k, err)
    assert err["pos"] <= 1.0, ("pos", err)
    return err
