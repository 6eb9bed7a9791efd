"""The FP64 network restatement (oracle/mpnn_oracle.py) checked on its own: its analytic
gradient against central finite differences of its loss, its feature definitions, and the
output heads' meaning (a constant acceleration gives O_v = O_x). CPU only."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import mpnn_oracle as MO


def small_frame(seed: int, n: int = 40):
    rng = np.random.default_rng(seed)
    h, c, dt = 0.02, 44.72, 1e-4
    pos = rng.uniform(0.0, 0.04, (n, 3))
    d = np.linalg.norm(pos[:, None, :] - pos[None, :, :], axis=-1)
    nb = np.full((n, MO.K), -1, dtype=np.int64)
    cnt = np.zeros(n, dtype=np.int64)
    for i in range(n):
        js = [j for j in np.argsort(d[i]) if j != i and d[i, j] < h][:MO.K]
        cnt[i] = len(js)
        nb[i, :len(js)] = js
    vel = rng.normal(0.0, 1.0, (n, 3))
    rho = rng.uniform(3900.0, 20000.0, n)
    e, mask, nf = MO.features(pos, vel, rho, nb, cnt, h, c, 3916.7, 1000.0, 3000.0, dt)
    target = rng.normal(0.0, 0.05, (n, MO.FO))
    return e, mask, nf, nb, target


def test_layout_size():
    assert MO.n_params() == len(MO.init_params(0))
    assert MO.FO == 6 and MO.FN == 9 and MO.FE == 14


def test_features():
    e, mask, nf, nb, _ = small_frame(1)
    assert np.all(e[~mask] == 0.0)
    r = e[..., 6]
    q = e[..., 7]
    assert np.all(r[mask] < 1.0) and np.allclose(q[mask], 1.0 - r[mask])
    # the spiky-gradient shape: |q^2 d / r| = q^2; the Laplacian shape: q u
    assert np.allclose(np.linalg.norm(e[..., 8:11], axis=-1)[mask], (q * q)[mask])
    assert np.allclose(e[..., 11:14][mask], (q[..., None] * e[..., 3:6])[mask])
    assert np.allclose(nf[:, 7], 1.0)
    assert np.allclose(nf[:, 8], 44.72 * 1e-4 / 0.02)


@pytest.mark.parametrize("seed", [2, 3])
def test_gradient_matches_finite_differences(seed):
    e, mask, nf, nb, target = small_frame(seed)
    flat = MO.init_params(seed).astype(np.float64)
    flat += np.random.default_rng(seed).normal(0.0, 0.05, flat.shape)  # non-zero biases too
    loss, _, grad = MO.loss_and_grad(flat, e, mask, nf, nb, target)
    rng = np.random.default_rng(100 + seed)
    off = 0
    for name, shape in MO.LAYOUT:
        size = int(np.prod(shape))
        for idx in rng.choice(size, size=min(6, size), replace=False):
            k = off + idx
            eps = 1e-6 * max(1.0, abs(flat[k]))
            up, dn = flat.copy(), flat.copy()
            up[k] += eps
            dn[k] -= eps
            num = (MO.loss_and_grad(up, e, mask, nf, nb, target)[0] -
                   MO.loss_and_grad(dn, e, mask, nf, nb, target)[0]) / (2 * eps)
            assert abs(num - grad[k]) <= 1e-5 * max(1e-3, abs(num)) + 1e-9, (name, idx, num, grad[k])
        off += size


def test_zero_network_outputs_zero():
    e, mask, nf, nb, _ = small_frame(4)
    out, _ = MO.forward(np.zeros(MO.n_params()), e, mask, nf, nb)
    assert np.all(out == 0.0)


def test_heads_of_a_constant_acceleration_agree():
    """For a_0 = a_1 = a_2 = a_3 = a the two target heads are equal (a / A), and the macro-step
    update reproduces 4 symplectic sub-steps exactly."""
    a, A, dt = np.array([3.0, -9.81, 0.5]), 1e5, 1e-4
    o_v = (4 * a) / (4 * A)
    o_x = (4 * a + 3 * a + 2 * a + a) / (10 * A)
    assert np.allclose(o_v, o_x)
    x, v = np.array([0.1, 0.2, 0.3]), np.array([1.0, 0.0, -2.0])
    xs, vs = x.copy(), v.copy()
    for _ in range(4):
        vs = vs + dt * a
        xs = xs + dt * vs
    assert np.allclose(vs, v + 4 * dt * A * o_v, rtol=0, atol=1e-15)
    assert np.allclose(xs, x + 4 * dt * v + 10 * dt * dt * A * o_x, rtol=0, atol=1e-15)
