"""Snapshot and trajectory files: the format restated here in numpy (a file written by this test
is read by the library and the other way round), checksum and corruption handling on the CPU;
save -> load -> continue bit for bit against an uninterrupted run, batched scenes and
trajectories on the GPU."""
from __future__ import annotations

import numpy as np
import pytest

M64 = (1 << 64) - 1


def fnv_words(b: bytes) -> int:
    if len(b) % 8:
        b = b + bytes(8 - len(b) % 8)
    h = 0xcbf29ce484222325
    for w in np.frombuffer(b, dtype="<u8").tolist():
        h = ((h ^ w) * 0x100000001b3) & M64
    return h


def write_snapshot(path, params_list, counts, particles, steps, seed, order=None):
    """An independent writer of the documented format."""
    table = b"".join(bytes(p) for p in params_list) + np.asarray(counts, "<u4").tobytes()
    table += bytes((-len(table)) % 64)
    recs = particles.tobytes() + (np.asarray(order, "<u4").tobytes() if order is not None else b"")
    head = np.zeros(1, dtype=[("magic", "S8"), ("version", "<u4"), ("hb", "<u4"), ("n", "<u8"), ("sc", "<u4"),
                              ("r0", "<u4"), ("steps", "<u8"), ("seed", "<u8"), ("sum", "<u8"), ("r1", "<u8")])
    head["magic"], head["version"], head["hb"] = b"NPRSPHS1", 1, 64
    head["r0"] = 1 if order is not None else 0  # flags: bit 0 = slot order present
    head["n"], head["sc"], head["steps"], head["seed"] = len(particles), len(params_list), steps, seed
    head["sum"] = fnv_words(table + recs)
    with open(path, "wb") as f:
        f.write(head.tobytes() + table + recs)


def test_checksum_matches_restatement(sph):
    rng = np.random.default_rng(0)
    for size in (0, 1, 7, 8, 9, 64, 1000):
        b = rng.integers(0, 256, size, dtype=np.uint8).tobytes()
        assert sph.checksum64(b) == fnv_words(b) if size else True


def test_library_reads_a_file_written_to_the_format(sph, tmp_path):
    sc = sph.dam_break(8, 8, 8, seed=4)
    path = tmp_path / "s.snap"
    write_snapshot(path, [sc.params], [len(sc.particles)], sc.particles, steps=17, seed=99)
    assert sph.snapshot_info(path) == {"n": 512, "scenes": 1, "steps": 17, "seed": 99}
    assert sph.snapshot_verify(path)
    r = sph.read_snapshot(path)
    assert r["steps"] == 17 and r["seed"] == 99 and list(r["counts"]) == [512]
    assert bytes(r["params"][0]) == bytes(sc.params)
    assert np.array_equal(r["particles"], sc.particles)


def test_slot_order_section(sph, tmp_path):
    sc = sph.dam_break(8, 8, 8, seed=4)
    order = np.random.default_rng(1).permutation(len(sc.particles)).astype(np.uint32)
    path = tmp_path / "o.snap"
    write_snapshot(path, [sc.params], [len(sc.particles)], sc.particles, steps=3, seed=1, order=order)
    assert sph.snapshot_verify(path)
    r = sph.read_snapshot(path)
    assert np.array_equal(r["slot_order"], order) and np.array_equal(r["particles"], sc.particles)
    raw = bytearray(path.read_bytes())
    raw[-3] ^= 0x10  # the order section is covered by the checksum
    bad = tmp_path / "bad.snap"
    bad.write_bytes(bytes(raw))
    assert not sph.snapshot_verify(bad)


def test_corrupt_or_truncated_files_are_refused(sph, tmp_path):
    sc = sph.dam_break(8, 8, 8, seed=5)
    path = tmp_path / "s.snap"
    write_snapshot(path, [sc.params], [len(sc.particles)], sc.particles, steps=0, seed=0)
    raw = bytearray(path.read_bytes())
    bad = tmp_path / "bad.snap"
    raw[64 + 128 + 200] ^= 0x01  # one bit of one record
    bad.write_bytes(bytes(raw))
    assert not sph.snapshot_verify(bad)
    short = tmp_path / "short.snap"
    short.write_bytes(path.read_bytes()[:-64])
    assert not sph.snapshot_verify(short)
    wrong = tmp_path / "wrong.snap"
    wrong.write_bytes(b"NPRSPHX1" + path.read_bytes()[8:])
    assert not sph.snapshot_verify(wrong)
    with pytest.raises(RuntimeError):
        sph.snapshot_info(wrong)


@pytest.mark.gpu
def test_save_load_continues_bit_for_bit(sph, gpu, tmp_path):
    sc = sph.dam_break(16, 32, 32, seed=6)
    n = len(sc.particles)
    path = tmp_path / "run.snap"
    with sph.Sim(sc.params, n_max=n) as a:
        a.upload(sc.particles)
        a.step(25)
        a.save(path, seed=6)
        saved = a.download()
        a.step(25)
        end_a = a.download()
        steps_a = a.steps
    assert sph.snapshot_verify(path)
    assert sph.snapshot_info(path)["steps"] == 25
    assert sph.read_snapshot(path)["slot_order"] is not None
    with sph.Sim.from_snapshot(path) as b:
        assert b.steps == 25
        assert np.array_equal(b.download(), saved)  # every field, rho and pres included
        b.step(25)
        end_b = b.download()
        assert b.steps == steps_a
    assert np.array_equal(end_a["pos"], end_b["pos"]) and np.array_equal(end_a["vel"], end_b["vel"])


@pytest.mark.gpu
def test_batched_snapshot_round_trip(sph, gpu, tmp_path):
    plist, counts, parts = sph.batched_scenes(6, seed=8, n_lo=2000, n_hi=6000)
    path = tmp_path / "batch.snap"
    with sph.Sim(plist, counts=counts) as a:
        a.upload(parts)
        a.step(5)
        a.save(path)
        saved = a.download()
    r = sph.read_snapshot(path)
    assert list(r["counts"]) == list(counts)
    assert [bytes(p) for p in r["params"]] == [bytes(p) for p in plist]
    assert np.array_equal(r["particles"], saved)
    with sph.Sim.from_snapshot(path) as b:
        assert b.n_scene == len(counts)
        assert np.array_equal(b.download(), saved)


@pytest.mark.gpu
def test_trajectory_frames_are_the_states(sph, gpu, tmp_path):
    sc = sph.dam_break(8, 16, 16, seed=9)
    path = tmp_path / "run.traj"
    states = []
    with sph.Sim(sc.params, n_max=len(sc.particles)) as sim:
        sim.upload(sc.particles)
        with sph.Trajectory(sim, path, seed=9) as tr:
            for _ in range(4):
                sim.step(3)
                tr.append(sim)
                states.append((sim.steps, sim.download()))
            assert tr.frames == 4
    t = sph.read_trajectory(path)
    assert t["seed"] == 9 and len(t["frames"]) == 4
    for (step, recs), (s_ref, ref) in zip(t["frames"], states):
        assert step == s_ref
        assert np.array_equal(recs, ref)
