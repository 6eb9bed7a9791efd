"""The BF16 tensor-core GEMM (tcgen05, FP32 accumulation in TMEM) that the training passes of
the learned macro-step use, against a float64 product of the same bf16-rounded operands.
FP32 accumulation of K products: |D - D64| <= 1e-5 * sum_k |a_ik b_jk| (with room to spare)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,n,k,splits", [(128, 64, 64, 1), (300, 16, 16, 1), (200, 80, 144, 1),
                                          (64, 144, 128, 1), (257, 128, 80, 1), (80, 64, 4096, 8)])
def test_tc_gemm_matches_float64(sph, gpu, m, n, k, splits):
    rng = np.random.default_rng(m * 7 + n * 3 + k)
    a = sph.to_bf16_bits(rng.normal(size=(m, k)).astype(np.float32))
    b = sph.to_bf16_bits(rng.normal(size=(n, k)).astype(np.float32))
    af = sph.bf16_bits_to_f32(a).astype(np.float64)
    bf = sph.bf16_bits_to_f32(b).astype(np.float64)
    d = sph.tc_gemm(a, b, splits).astype(np.float64)
    got = d.sum(axis=0)
    ref = af @ bf.T
    scale = np.abs(af) @ np.abs(bf).T
    err = np.abs(got - ref) / scale
    assert err.max() < 1e-5, (err.max(), np.unravel_index(err.argmax(), err.shape))


def test_tc_gemm_rejects_bad_shapes(sph):
    a = np.zeros((16, 24), np.uint16)
    with pytest.raises(sph.SphError):
        sph.tc_gemm(a, np.zeros((16, 24), np.uint16))  # k not a multiple of 16
    with pytest.raises(sph.SphError):
        sph.tc_gemm(np.zeros((16, 16), np.uint16), np.zeros((24, 16), np.uint16))  # n not a multiple of 16
