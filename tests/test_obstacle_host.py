"""Static obstacles, host side: the OBJ reader (sph_obj_read), the icosphere mesh, and the
FP64 restatements in oracle/ of the mesh signed distance field and of the collision rule.
No GPU needed."""
from __future__ import annotations

import numpy as np
import pytest


def test_obj_read_faces_and_index_forms(sph, tmp_path):
    path = tmp_path / "m.obj"
    path.write_text(
        "# a unit square, a triangle and a pentagon\n"
        "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\n"
        "vt 0 0\nvn 0 0 1\n"
        "f 1/1/1 2/1/1 3/1/1 4/1/1\n"      # quad -> fan (0 1 2) (0 2 3)
        "v 0 0 1\nv 1 0 1\nv 0 1 1\n"
        "f -3 -2 -1\n"                      # negative indices: the last three vertices
        "f 5//1 6//1 3//1 4//1 7//1  # pentagon\n"
        "o ignored\ns off\n")
    v, t = sph.obj_read(path)
    assert v.shape == (7, 3) and t.shape == (6, 3)
    np.testing.assert_array_equal(v[4], [0, 0, 1])
    np.testing.assert_array_equal(t, [[0, 1, 2], [0, 2, 3], [4, 5, 6], [4, 5, 2], [4, 2, 3], [4, 3, 6]])


def test_obj_read_errors(sph, tmp_path):
    import ctypes as C

    with pytest.raises(sph.SphError):
        sph.obj_read(tmp_path / "missing.obj")
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 4\n")  # index past the vertices read so far
    with pytest.raises(sph.SphError):
        sph.obj_read(bad)
    ok = tmp_path / "ok.obj"
    ok.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    nv, nt = C.c_uint32(2), C.c_uint32(1)
    v = np.zeros((3, 3), np.float32)
    t = np.zeros((1, 3), np.uint32)
    rc = sph.lib.sph_obj_read(str(ok).encode(), v.ctypes.data, C.byref(nv), t.ctypes.data, C.byref(nt))
    assert rc == sph.ERR_CAPACITY and (nv.value, nt.value) == (3, 1)


def test_icosphere_round_trip_and_orientation(sph, tmp_path):
    v, t = sph.icosphere(0.1, (0.5, 0.5, 0.5), 2)
    assert v.shape == (162, 3) and t.shape == (320, 3)
    np.testing.assert_allclose(np.linalg.norm(v.astype(np.float64) - 0.5, axis=1), 0.1, rtol=1e-6)
    a, b, c = (v[t[:, k]].astype(np.float64) for k in range(3))
    volume = np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0
    assert 0.9 * 4.0 / 3.0 * np.pi * 0.1 ** 3 < volume < 4.0 / 3.0 * np.pi * 0.1 ** 3  # outward, inscribed
    sph.write_obj(tmp_path / "s.obj", v, t)
    v2, t2 = sph.obj_read(tmp_path / "s.obj")
    np.testing.assert_array_equal(v2, v)
    np.testing.assert_array_equal(t2, t)


def test_mesh_sdf_restatement_against_the_sphere(sph, orc):
    v, t = sph.icosphere(0.1, (0.5, 0.5, 0.5), 3)
    g = np.linspace(0.3, 0.7, 11)
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    phi = orc.mesh_sdf(v, t, pts)
    exact = np.linalg.norm(pts - 0.5, axis=1) - 0.1
    # the inscribed mesh lies within r (1 - cos(edge angle)) < 1e-3 of the sphere
    assert np.max(np.abs(phi - exact)) < 1e-3
    far = np.abs(exact) > 2e-3
    assert np.array_equal(np.sign(phi[far]), np.sign(exact[far]))
    # a vertex, an edge midpoint and a face centre of the mesh are at distance 0
    a, b, c = v[t[0]].astype(np.float64)
    on = np.array([a, 0.5 * (a + b), (a + b + c) / 3.0])
    assert np.max(np.abs(orc.mesh_sdf(v, t, on))) < 1e-12


def test_obstacle_rule_oracle(sph, orc):
    """The FP64 rule on a sampled sphere: a particle inside moves out to the surface along the
    normal and keeps -damping of its inward normal velocity; one outside is untouched."""
    p = sph.workload_params(lower=(0.0, 0.0, 0.0), upper=(1.0, 1.0, 1.0))
    n_s, spacing = 41, 0.025
    g = np.arange(n_s) * spacing
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    sdf = (np.sqrt((x - 0.5) ** 2 + (y - 0.5) ** 2 + (z - 0.5) ** 2) - 0.2).astype(np.float32)
    pos = np.array([[0.5, 0.68, 0.5], [0.5, 0.9, 0.5]])
    vel = np.array([[0.3, -2.0, 0.0], [0.0, -2.0, 0.0]])
    x1, v1, phi = orc.obstacle_f64(p, sdf, (0.0, 0.0, 0.0), spacing, pos, vel)
    assert phi[0] < 0.0 < phi[1]
    assert abs(np.linalg.norm(x1[0] - 0.5) - 0.2) < 1e-3  # on the sampled surface
    # the normal at the top is (0, 1, 0) up to the O(spacing^2) error of the sampled gradient
    assert x1[0, 1] > pos[0, 1] and abs(x1[0, 0] - 0.5) < 1e-5 and abs(x1[0, 2] - 0.5) < 1e-5
    np.testing.assert_allclose(v1[0], [0.3, 2.0 * p.damping, 0.0], atol=2e-3)
    np.testing.assert_array_equal(x1[1], pos[1])
    np.testing.assert_array_equal(v1[1], vel[1])
