"""sph_reduce_aos_noalloc: FP64 diagnostics of a caller-owned device buffer with no allocation.

Callers that cannot allocate device memory when they need the diagnostics (a frame loop
with a fixed GPU memory budget, a plugin host that owns every buffer) pass their particle buffer and an output buffer; the scratch of the
reduction is a fixed device array inside the library. This checks it through the C ABI
against the context-based sph_reduce on the same state, on two calls in a row.

This file sorts last so that a run stopping at its first failure has run every other
test before it; it also passes on its own in a fresh process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = 12


def noalloc_sums(sph, dev_ptr: int, n: int, params, stream_ptr: int = 0) -> np.ndarray:
    import torch

    out = torch.zeros(FIELDS, dtype=torch.float64, device="cuda")
    rc = sph.lib.sph_reduce_aos_noalloc(C.c_void_p(dev_ptr), n, C.byref(params), C.c_void_p(out.data_ptr()),
                                        C.c_void_p(stream_ptr))
    assert rc == sph.OK, rc
    torch.cuda.synchronize()
    return out.cpu().numpy()


def as_diag(s: np.ndarray) -> dict:
    cnt = s[10]
    return {"momentum": s[0:3], "kinetic_energy": s[3], "potential_energy": s[4], "mean_rho": s[5] / cnt,
            "min_rho": s[6], "max_rho": s[7], "mean_abs_rho_dev": s[8] / cnt, "nonfinite": int(s[9]),
            "n": int(s[9] + s[10])}


def test_noalloc_matches_sph_reduce_twice(sph, gpu):
    import torch

    sc = sph.dam_break(32, 64, 64, seed=14)  # 131,072 particles: 32 CTAs of partials
    n = len(sc.particles)
    dev = torch.zeros(n * 64, dtype=torch.uint8, device="cuda")
    with sph.Sim(sc.params, n_max=n) as sim:
        sim.upload(sc.particles)
        for _ in range(2):  # two calls in a row: the shared scratch keeps the last call's rows
            sim.step(7)
            ref = sim.reduce()
            sim.download_device(dev.data_ptr(), n)
            sim.synchronize()
            got = as_diag(noalloc_sums(sph, dev.data_ptr(), n, sc.params))
            np.testing.assert_allclose(got["momentum"], list(ref.momentum), rtol=1e-12, atol=1e-12)
            for k in ("kinetic_energy", "potential_energy", "mean_rho", "mean_abs_rho_dev"):
                assert got[k] == pytest.approx(getattr(ref, k), rel=1e-12, abs=1e-12), k
            assert got["min_rho"] == ref.min_rho and got["max_rho"] == ref.max_rho
            assert got["nonfinite"] == ref.nonfinite and got["n"] == ref.n == n


def test_noalloc_smaller_call_after_larger_and_limits(sph, gpu):
    import torch

    p = sph.default_params()
    rng = np.random.default_rng(4)
    big = sph.empty_particles(20000)
    big["vel"][:, :3] = rng.normal(size=(20000, 3)).astype(np.float32)
    big["extras"][:, 0] = rng.uniform(900, 1100, 20000).astype(np.float32)
    dev = torch.from_numpy(big.view(np.uint8).copy()).cuda()
    a = noalloc_sums(sph, dev.data_ptr(), 20000, p)
    b = noalloc_sums(sph, dev.data_ptr(), 5, p)  # fewer rows than the previous call left behind
    m = float(np.float32(p.mass))
    np.testing.assert_allclose(a[0:3], m * big["vel"][:, :3].astype(np.float64).sum(0), rtol=1e-12)
    np.testing.assert_allclose(b[0:3], m * big["vel"][:5, :3].astype(np.float64).sum(0), rtol=1e-12)
    assert b[10] == 5 and a[10] == 20000
    out = torch.zeros(FIELDS, dtype=torch.float64, device="cuda")
    rc = sph.lib.sph_reduce_aos_noalloc(C.c_void_p(dev.data_ptr()), 4_194_305, C.byref(p),
                                        C.c_void_p(out.data_ptr()), None)
    assert rc == sph.ERR_CAPACITY
    assert sph.lib.sph_reduce_aos_noalloc(None, 5, C.byref(p), C.c_void_p(out.data_ptr()), None) == sph.ERR_INVALID_ARG
