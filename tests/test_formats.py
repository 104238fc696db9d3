"""Output formats: SEMTRC01 traces (trace-major float32 + JSON header) and SEMSNP01 snapshots
(one x-z plane), written by the library and read back by it and by the numpy readers."""
import json

import numpy as np
import pytest


def test_traces_round_trip(semgb_lib, tmp_path):
    semgb = semgb_lib
    from semgb import formats
    rng = np.random.default_rng(3)
    tr = rng.standard_normal((57, 9)).astype(np.float32)
    rec = rng.uniform(0, 100, (9, 3)).astype(np.float32)
    src = np.array([[50.0, 40.0, 30.0]], np.float32)
    p = tmp_path / "shot0.semtrc"
    semgb.write_traces(p, tr, 1.5e-4, rec, src, extra_json='{"shot": 0, "model": "c2"}')
    back, dt = semgb.read_traces(p)
    assert np.array_equal(back, tr) and dt == np.float32(1.5e-4)
    h, back2 = formats.read_traces(p)
    assert np.array_equal(back2, tr)
    assert h["n_traces"] == 9 and h["n_samples"] == 57 and h["order"] == "trace-major"
    assert np.allclose(h["receivers"], rec) and np.allclose(h["sources"], src)
    assert h["extra"] == {"shot": 0, "model": "c2"}
    raw = p.read_bytes()
    n = int.from_bytes(raw[8:16], "little")
    off = (16 + n + 63) // 64 * 64
    # trace-major on disk: the first n_samples values are receiver 0's series
    first = np.frombuffer(raw, "<f4", count=57, offset=off)
    assert np.array_equal(first, tr[:, 0])
    assert len(raw) == off + tr.size * 4
    json.loads(raw[16:16 + n])


def test_traces_reject_bad_files(semgb_lib, tmp_path):
    semgb = semgb_lib
    p = tmp_path / "bad.semtrc"
    p.write_bytes(b"NOTATRACEFILE" + bytes(100))
    with pytest.raises(semgb.SemError):
        semgb.read_traces(p)
    # truncated data
    q = tmp_path / "short.semtrc"
    semgb.write_traces(q, np.ones((10, 4), np.float32), 1e-3)
    q.write_bytes(q.read_bytes()[:-8])
    with pytest.raises(semgb.SemError):
        semgb.read_traces(q)


@pytest.mark.gpu
def test_snapshot_is_the_plane_of_the_level(semgb_lib, cuda_device, tmp_path):
    semgb = semgb_lib
    from semgb import formats
    from semgb import workloads as W
    wl = W.small_random(6, 5, 4, 3, 25, seed=21, nsrc=1, nrec=4)
    mesh, s = semgb.solver_from_workload(wl, semgb.KERNEL_STENCIL)
    s.step(25)
    nx, ny, nz = wl.ex * 3 + 1, wl.ey * 3 + 1, wl.ez * 3 + 1
    p = s.pressure().reshape(ny, nz, nx)
    f = tmp_path / "snap.semsnp"
    s.write_snapshot(f)
    plane, y = semgb.read_snapshot(f)
    assert y == ny // 2 - 1
    assert np.array_equal(plane, p[y])
    h, plane2 = formats.read_snapshot(f)
    assert np.array_equal(plane2, p[y]) and h["step"] == 25 and len(h["x"]) == nx and len(h["z"]) == nz
    s.write_snapshot(f, semgb.LEVEL_PREVIOUS, 2)
    plane3, y3 = semgb.read_snapshot(f)
    assert y3 == 2
    assert np.array_equal(plane3, s.pressure(semgb.LEVEL_PREVIOUS).reshape(ny, nz, nx)[2])
