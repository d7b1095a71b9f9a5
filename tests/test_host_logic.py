"""Host-side logic on the CPU: trajectory trim rule, shadow-pass row
selection, request packing, workload constants, metrics, the synthetic
snapshot, and the replica helpers over a 2-rank gloo group."""

import ctypes
import os

import numpy as np
import pytest

from conftest import golden


def test_trimmed_rows_matches_reference_rule(orc):
    from mahakala_gb300.geodesics import trimmed_rows
    N = 100
    for K in (np.array([3, 7, 5]), np.array([0, 0]), np.array([99, 2]), np.array([100, 4]), np.array([1]),
              np.array([98])):
        assert trimmed_rows(K, N) == orc.trimmed_rows(K, N)
    # every ray stopped at row F = max K: F + 2 rows; none: N rows
    assert trimmed_rows(np.array([3, 7, 5]), N) == 9
    assert trimmed_rows(np.array([100, 4]), N) == N
    assert trimmed_rows(np.array([0, 0]), N) == N
    assert trimmed_rows(np.array([99, 2]), N) == N


def test_trim_rule_on_reference_fixture():
    from mahakala_gb300.geodesics import trimmed_rows
    d = golden("integrator")
    for c in range(3):
        N = int(d[f"case{c}_params"][4])
        # nsteps per ray is K of that ray (stopped rays: K < N)
        assert trimmed_rows(d[f"case{c}_nsteps"], N) == int(d[f"case{c}_rows"])


def test_request_struct_layout():
    from mahakala_gb300 import _lib
    assert ctypes.sizeof(_lib.Request) == 304
    assert ctypes.sizeof(_lib.SnapshotView) == 128
    assert ctypes.sizeof(_lib.MeshDesc) == 168
    assert _lib.Request.ray_offset.offset == 264
    assert _lib.Request.rows.offset == 296


def test_mass_scale_interpolation():
    from mahakala_gb300 import configs
    assert configs.mass_scale_for(1.0) == pytest.approx(3e26)
    assert configs.mass_scale_for(10.0) == pytest.approx(3e27)
    assert configs.mass_scale_for(40.0) == pytest.approx(8e28)
    xs = [1, 2, 5, 10, 20, 40, 60, 80]
    ys = [configs.mass_scale_for(x) for x in xs]
    assert all(b > a for a, b in zip(ys, ys[1:]))
    assert configs.RENDER_256.mass_scale == configs.MASS_SCALE_256


def test_metrics():
    from mahakala_gb300 import _lib, metrics
    ref = np.array([[1.0, 2.0], [0.0, 4.0]])
    img = ref * (1 + 1e-3)
    assert metrics.flux_rel_err(img, ref) == pytest.approx(1e-3)
    assert metrics.max_pixel_rel_err(img, ref) == pytest.approx(1e-3)
    # the zero pixel is compared against the floor 1e-4 * max
    img2 = ref.copy()
    img2[1, 0] = 4e-6
    assert metrics.max_pixel_rel_err(img2, ref) == pytest.approx(1e-2)
    st = np.full((10, 10), _lib.MK_RAY_ESCAPED)
    st[3:7, 3:7] = _lib.MK_RAY_CAPTURED
    assert metrics.shadow_diameter(st, 10.0) == pytest.approx(2 * np.sqrt(16 / np.pi))


def test_synthetic_snapshot_properties():
    from mahakala_gb300.grmhd.synthetic import make_synthetic_snapshot
    a = make_synthetic_snapshot(nblocks=2, cells_per_block=8, extent=20.0, bhspin=0.9, seed=5)
    b = make_synthetic_snapshot(nblocks=2, cells_per_block=8, extent=20.0, bhspin=0.9, seed=5)
    c = make_synthetic_snapshot(nblocks=2, cells_per_block=8, extent=20.0, bhspin=0.9, seed=6)
    assert np.array_equal(a.uov, b.uov) and not np.array_equal(a.uov, c.uov)
    assert a.uov.dtype == np.float32 and a.uov.shape == (5, 8, 8, 8, 8) and a.B.shape == (3, 8, 8, 8, 8)
    # exact cell geometry: dx = 40/16 = 2.5
    assert np.all(a.x1v[:, 1] - a.x1v[:, 0] == 2.5)
    assert np.array_equal(a.x1f[:, -1] - a.x1f[:, 0], np.full(8, 20.0))
    # excised cells inside the horizon are zero, the rest positive density
    assert (a.uov[0] > 0).mean() > 0.9
    assert np.all(a.uov[0] >= 0) and np.all(np.isfinite(a.uov))
    # the snapshot in the fixture is this generator's output
    d = golden("snapshot")
    assert np.array_equal(d["uov"], a.uov)


def test_ray_range_partitions():
    from mahakala_gb300.replicas import ray_range
    for total in (0, 1, 7, 65536):
        for world in (1, 2, 3, 8):
            spans = [ray_range(total, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == total
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            assert max(b - a for a, b in spans) - min(b - a for a, b in spans) <= 1


def _replica_worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from mahakala_gb300.replicas import gather_ranges, max_over_ranks, ray_range
    total = 11
    a, b = ray_range(total, rank, world)
    local = torch.arange(a, b, dtype=torch.float64) * 10
    full = gather_ranges(local, total)
    t = max_over_ranks(1.0 + rank)
    out.put((rank, full.tolist(), t))
    dist.destroy_process_group()


def test_replicas_over_gloo():
    import socket

    import torch.multiprocessing as mp
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    for rank, full, t in res:
        assert full == [10.0 * i for i in range(11)]
        assert t == 2.0


@pytest.mark.parametrize("case", [0, 1])
def test_mesh_tables_multilevel(case):
    """Finest-level block table covers the refined mesh once per cell, each
    block over exactly its own span; the blocks flagged for a binary64 copy
    include every block whose reference ghost fill produced a value that is
    not a float32 value (a fine-to-coarse mean)."""
    from conftest import amr_arrays, golden
    from mahakala_gb300.grmhd.athenak import mesh_tables
    arrs = amr_arrays(case)
    t = mesh_tables(arrs)
    table = t["table"]
    assert (table >= 0).all()
    lv = np.asarray(arrs.Levels)
    counts = np.bincount(table.ravel(), minlength=len(lv))
    assert np.array_equal(counts, 8 ** (lv.max() - lv))      # a level-l block spans 2^(L-l) cells per axis
    ref = golden("amr")[f"case{case}_all_meshblocks"]
    inexact = np.any((ref.astype(np.float32).astype(np.float64) != ref).reshape(len(lv), -1), axis=1)
    assert np.all(t["block64"][inexact] >= 0)
    assert t["n64"] == int((t["block64"] >= 0).sum())
    keys = t["keys"]
    assert np.all(np.diff(keys) > 0)
