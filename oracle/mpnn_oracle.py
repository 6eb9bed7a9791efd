"""FP64 restatement of the learned message-passing macro-step. TEST INFRASTRUCTURE ONLY.

Only tests/ and the CPU legs of bench.py may import this module. It defines, in plain
numpy float64, the network the GPU kernels of npr-sph_gb300/csrc/sph_mpnn.cu compute
(FP32 training kernels, BF16 tensor-core inference), so their forward pass and gradients
can be checked against it.

The network has no counterpart in the reference (NPR-SPH has no learned component). It
predicts, per particle, the mean accelerations of the next 4 plain steps (a macro-step of
4*dt) from the particle's neighbourhood:

  edge features  e_ij = [ d (3), u (3), r/h, q, q^2 d / (r/h) (3), q u (3) ]        (14)
                 d = (x_j-x_i)/h, u = (v_j-v_i)/c, q = 1 - r/h; the spiky-gradient and
                 viscosity-Laplacian shapes of force_comp.glsl:59-60 (the first is 0 at r = 0)
  node features  n_i  = [ v_i/c (3), rho_i/rho_self - 1, (rho_i-rho0)/rho_self,
                          log10(mu)/4, cnt_i/K, 1, c*dt/h ]                         (9)
  round 1   Z1_ij = e_ij We1 + be1,  M1_i = sum_j relu(Z1_ij) / K
            Y1_i  = [M1_i, n_i] Wn1 + bn1,  H1_i = relu(Y1_i),  P_i = H1_i Wp
  round 2   Z2_ij = e_ij We2 + P_j + be2,  M2_i = sum_j relu(Z2_ij) / K
            Y2_i  = [M2_i, H1_i] Wn2 + bn2,  H2_i = relu(Y2_i)
  output    O_i = H2_i Wo + bo = (O_v, O_x)                                          (6)
            O_v = (a_0 + a_1 + a_2 + a_3) / (4A),  O_x = (4 a_0 + 3 a_1 + 2 a_2 + a_3) / (10A)

with a_s the SPH acceleration F/rho of plain sub-step s and A = k/h; the macro-step is then
v' = v + 4 dt A O_v, x' = x + 4 dt v + 10 dt^2 A O_x (exact for 4 symplectic sub-steps).
j runs over the (at most K = 32) nearest neighbours of i with r < h, i excluded;
c = sqrt(k) is the sound speed of the linear EOS; rho_self = m*315/(64*pi*h^3).
Loss: mean over particles of |O_i - target_i|^2.
"""
from __future__ import annotations

import numpy as np

K = 32
W = 64
FE = 14
FN = 9
FO = 6

# Flat parameter layout (float32 on the GPU), in this order.
LAYOUT = [("We1", (FE, W)), ("be1", (W,)), ("Wn1", (W + FN, W)), ("bn1", (W,)), ("Wp", (W, W)),
          ("We2", (FE, W)), ("be2", (W,)), ("Wn2", (2 * W, W)), ("bn2", (W,)), ("Wo", (W, FO)), ("bo", (FO,))]


def n_params() -> int:
    return sum(int(np.prod(s)) for _, s in LAYOUT)


def unpack(flat: np.ndarray) -> dict:
    out, o = {}, 0
    for name, shape in LAYOUT:
        size = int(np.prod(shape))
        out[name] = flat[o:o + size].reshape(shape)
        o += size
    return out


def pack(p: dict) -> np.ndarray:
    return np.concatenate([np.asarray(p[name], dtype=np.float64).reshape(-1) for name, _ in LAYOUT])


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation (the GPU trainer starts from the same flat vector)."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, shape in LAYOUT:
        if name.startswith("W"):
            fan_in = shape[0]
            scale = np.sqrt(2.0 / fan_in) if name != "Wo" else 0.1 / np.sqrt(fan_in)
            p[name] = rng.normal(0.0, scale, shape)
        else:
            p[name] = np.zeros(shape)
    return pack(p).astype(np.float32)


def features(pos, vel, rho, nb, cnt, h, c, rho_self, rho0, mu, dt):
    """Edge features e (n, K, 14) with padded edges zeroed, edge mask (n, K), node features (n, 9)."""
    pos = np.asarray(pos, np.float64)
    vel = np.asarray(vel, np.float64)
    n = len(pos)
    mask = np.arange(K)[None, :] < np.asarray(cnt)[:, None]
    j = np.where(mask, nb, 0)
    d = (pos[j] - pos[:, None, :]) / h
    u = (vel[j] - vel[:, None, :]) / c
    r = np.sqrt((d * d).sum(-1))
    q = 1.0 - r
    sg = np.where(r > 0.0, q * q / np.where(r > 0.0, r, 1.0), 0.0)
    e = np.concatenate([d, u, r[..., None], q[..., None], sg[..., None] * d, q[..., None] * u], axis=-1)
    e = np.where(mask[..., None], e, 0.0)
    rho = np.asarray(rho, np.float64)
    nf = np.zeros((n, FN))
    nf[:, 0:3] = vel / c
    nf[:, 3] = rho / rho_self - 1.0
    nf[:, 4] = (rho - rho0) / rho_self
    nf[:, 5] = np.log10(mu) / 4.0
    nf[:, 6] = np.asarray(cnt, np.float64) / K
    nf[:, 7] = 1.0
    nf[:, 8] = c * dt / h
    return e, mask, nf


def forward(flat, e, mask, nf, nb):
    p = unpack(np.asarray(flat, np.float64))
    relu = lambda x: np.maximum(x, 0.0)
    m = mask[..., None].astype(np.float64)
    Z1 = e @ p["We1"] + p["be1"]
    M1 = (relu(Z1) * m).sum(1) / K
    X1 = np.concatenate([M1, nf], axis=1)
    Y1 = X1 @ p["Wn1"] + p["bn1"]
    H1 = relu(Y1)
    P = H1 @ p["Wp"]
    j = np.where(mask, nb, 0)
    Z2 = e @ p["We2"] + P[j] + p["be2"]
    M2 = (relu(Z2) * m).sum(1) / K
    X2 = np.concatenate([M2, H1], axis=1)
    Y2 = X2 @ p["Wn2"] + p["bn2"]
    H2 = relu(Y2)
    O = H2 @ p["Wo"] + p["bo"]
    cache = dict(p=p, e=e, m=m, mask=mask, j=j, Z1=Z1, X1=X1, Y1=Y1, H1=H1, Z2=Z2, X2=X2, Y2=Y2, H2=H2)
    return O, cache


def loss_and_grad(flat, e, mask, nf, nb, target):
    """Mean squared error over particles and its gradient w.r.t. the flat parameters."""
    O, c = forward(flat, e, mask, nf, nb)
    n = len(O)
    diff = O - target
    loss = float((diff * diff).sum() / n)
    dO = 2.0 * diff / n
    p = c["p"]
    g = {}
    g["Wo"] = c["H2"].T @ dO
    g["bo"] = dO.sum(0)
    dY2 = (dO @ p["Wo"].T) * (c["Y2"] > 0)
    g["Wn2"] = c["X2"].T @ dY2
    g["bn2"] = dY2.sum(0)
    dX2 = dY2 @ p["Wn2"].T
    dM2, dH1 = dX2[:, :W], dX2[:, W:].copy()
    dZ2 = (dM2[:, None, :] / K) * (c["Z2"] > 0) * c["m"]
    g["We2"] = np.einsum("nkf,nko->fo", c["e"], dZ2)
    g["be2"] = dZ2.sum((0, 1))
    dP = np.zeros_like(c["H1"])
    np.add.at(dP, c["j"].reshape(-1), dZ2.reshape(-1, W))
    g["Wp"] = c["H1"].T @ dP
    dH1 += dP @ p["Wp"].T
    dY1 = dH1 * (c["Y1"] > 0)
    g["Wn1"] = c["X1"].T @ dY1
    g["bn1"] = dY1.sum(0)
    dM1 = (dY1 @ p["Wn1"].T)[:, :W]
    dZ1 = (dM1[:, None, :] / K) * (c["Z1"] > 0) * c["m"]
    g["We1"] = np.einsum("nkf,nko->fo", c["e"], dZ1)
    g["be1"] = dZ1.sum((0, 1))
    return loss, O, pack(g)


def adam_step(flat, grad, m, v, t, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update (t counts from 1); returns the new (flat, m, v)."""
    m = beta1 * m + (1 - beta1) * grad
    v = beta2 * v + (1 - beta2) * grad * grad
    mh = m / (1 - beta1 ** t)
    vh = v / (1 - beta2 ** t)
    return flat - lr * mh / (np.sqrt(vh) + eps), m, v
