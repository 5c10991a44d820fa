"""GPU batches (mtgl_batch_render): many contexts' frames rendered by one pipeline run.

A batched frame must come out exactly as the same frame rendered alone: against the CPU
oracle with the usual tolerance (depth and stencil bit-exact, colour within 1 LSB), and
against the plain per-context GPU path bit for bit. Covers every tile size, graph capture
and replay, the cost-ordered work queue, the capacity-overflow re-run, frames that flush
passes of their own before the batch, and contexts reused after a batch.
"""
import concurrent.futures as cf
import os

import numpy as np
import pytest

import feature_scenes as F
import harness
from mytinygl_gb300 import workloads as W
from mytinygl_gb300.scene import render

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    return harness.product()


@pytest.fixture(scope="module")
def oracle():
    return harness.oracle()


def small_uneven(n=20, seed=11):
    return W.uneven_batch(n, seed=seed, min_side=16, max_side=200, min_tri=20, max_tri=3000, tex_size=32)


def setup_frames(glib, scenes):
    """A context per scene with its resident part played; returns (contexts, frame streams)."""
    ctxs, streams = [], []
    for s in scenes:
        c = glib.context(s.width, s.height)
        k = W.frame_start(s)
        s.play(c, 0, k)
        c.finish()
        ctxs.append(c)
        streams.append(s.stream(k))
    return ctxs, streams


def read_all(ctxs):
    out = []
    for c in ctxs:
        col, dep, st = c.read()
        out.append((col, dep, st, c.glGetError()))
    return out


def batched(glib, scenes, rounds=1, **config):
    ctxs, streams = setup_frames(glib, scenes)
    b = glib.batch(**config)
    for _ in range(rounds):
        glib.play_many(ctxs, streams)
        b.render(ctxs)
    b.wait()
    out = read_all(ctxs)
    stats = b.stats()
    b.destroy()
    for c in ctxs:
        c.destroy()
    return out, stats


def plain(glib, scenes):
    ctxs, streams = setup_frames(glib, scenes)
    for c, s in zip(ctxs, streams):
        glib.play(c, s)
        c.finish()
    out = read_all(ctxs)
    for c in ctxs:
        c.destroy()
    return out


def assert_identical(a, b, names):
    for (ca, da, sa, ea), (cb, db, sb, eb), n in zip(a, b, names):
        assert ea == eb, n
        assert np.array_equal(ca, cb), f"{n}: colour differs at {(ca != cb).sum()} pixels"
        assert harness.depth_equal(da, db).all(), f"{n}: depth differs"
        assert np.array_equal(sa, sb), f"{n}: stencil differs"


@pytest.mark.parametrize("tile", [8, 16, 32])
def test_batch_matches_oracle(gpu, oracle, tile):
    scenes = small_uneven()
    got, stats = batched(gpu, scenes, tile_size=tile)
    assert stats["frames"] == len(scenes) and stats["batches"] == 1
    for s, g in zip(scenes, got):
        want = render(oracle, s)
        harness.assert_parity(harness.compare(want, g, harness.cleared_buffers(s)), color_tol=1, name=s.name)


@pytest.mark.parametrize("config", [dict(tile_size=8), dict(tile_size=16, use_graph=0),
                                    dict(tile_size=32, order_by_cost=0), dict(tile_size=16, ctas_per_sm=1)])
def test_batch_matches_plain_exactly(gpu, config):
    scenes = small_uneven(24, seed=12)
    got, _ = batched(gpu, scenes, **config)
    assert_identical(got, plain(gpu, scenes), [s.name for s in scenes])


def test_graph_replay(gpu):
    scenes = small_uneven(12, seed=13)
    got, stats = batched(gpu, scenes, rounds=4, tile_size=16)
    assert stats["batches"] == 4
    assert stats["graph_captures"] >= 1 and stats["graph_replays"] >= 2, stats
    assert_identical(got, plain(gpu, scenes), [s.name for s in scenes])


def test_capacity_overflow_reruns_exactly(gpu):
    scenes = small_uneven(10, seed=14)
    got, stats = batched(gpu, scenes, rounds=2, tile_size=16, record_factor=0.01, pair_factor=0.01)
    assert stats["overflow_reruns"] == 1, stats  # the second round uses the learned capacities
    assert_identical(got, plain(gpu, scenes), [s.name for s in scenes])


def test_feature_scenes_as_one_batch(gpu, oracle):
    """Whole feature scenes (resource uploads, mid-scene clears and flushes included) played
    onto their contexts; whatever each leaves pending is rendered by one batch."""
    names = ["blend", "stencil", "scissor_mask", "fog", "lighting_phong", "texture_modes", "depth_range",
             "clip_big", "display_lists", "vbo", "draw_pixels", "viewport", "culling"]
    scenes = [F.SCENES[n][0]() for n in names]
    ctxs = [gpu.context(s.width, s.height) for s in scenes]
    gpu.play_many(ctxs, [s.stream() for s in scenes])
    b = gpu.batch(tile_size=8)
    b.render(ctxs)
    got = read_all(ctxs)
    b.destroy()
    for s, g, c in zip(scenes, got, ctxs):
        harness.assert_parity(harness.compare(render(oracle, s), g, harness.cleared_buffers(s)), 1, s.name)
        c.destroy()


def test_context_reused_after_batch(gpu, oracle):
    """A context whose frame went through a batch keeps drawing without waiting: its next
    pass is ordered after the batch. The oracle replays the same calls on one context."""
    first, second = F.SCENES["blend"][0](), F.SCENES["zbuffer"][0]()
    others = small_uneven(5, seed=15)
    ctxs, streams = setup_frames(gpu, others)
    ctx = gpu.context(first.width, first.height)
    gpu.play(ctx, first.stream())
    b = gpu.batch(tile_size=16)
    gpu.play_many(ctxs, streams)
    b.render(ctxs + [ctx])
    gpu.play(ctx, second.stream())  # clears and draws again while the batch may still run
    c, d, s = ctx.read()
    got = (c, d, s, ctx.glGetError())
    b.destroy()
    ref = oracle.context(first.width, first.height)
    oracle.play(ref, first.stream())
    oracle.play(ref, second.stream())
    rc, rd, rs = ref.read()
    want = (rc, rd, rs, ref.glGetError())
    harness.assert_parity(harness.compare(want, got), 1, "reused")
    for x in ctxs + [ctx, ref]:
        x.destroy()


def test_render_read_with_direct_uploads(gpu):
    """Client-array frames through mtgl_batch_render_read over several rounds: the first
    round copies the frames' staged bytes into the batch's staging area, later rounds send
    them straight from each context's staging area (round three adds frames past the device
    copy's size, which then grows keeping what was sent). Colour copied out by the batch
    equals what the plain path renders, every round."""
    scenes = W.uneven_batch(18, seed=15, min_side=16, max_side=160, min_tri=20, max_tri=2500, tex_size=32,
                            use_vbo=False)
    want = plain(gpu, scenes)
    ctxs, streams = setup_frames(gpu, scenes)
    b = gpu.batch(tile_size=16)
    for k in (6, 6, 18, 18):
        hosts = [np.zeros((s.height, s.width), np.uint32) for s in scenes[:k]]
        gpu.play_many(ctxs[:k], streams[:k])
        b.render(ctxs[:k], colors=hosts)
        b.wait()
        for h, w, s in zip(hosts, want, scenes):
            assert np.array_equal(h, w[0]), f"{s.name} (batch of {k})"
    b.destroy()
    for c in ctxs:
        c.destroy()


def test_readback_kernel_destinations(gpu):
    """Colour read-back into page-locked host memory runs as kernels writing the host buffers
    (16-byte stores where both ends are aligned, 4-byte ones elsewhere); pageable
    destinations are copied. Frames with odd sides, a page-locked destination 4 bytes off
    alignment and pageable ones in one batch: every destination equals the plain path's
    colour, with read-back kernels on and off, and the kernel mode launches one kernel more
    than the copy mode for the same run."""
    torch = pytest.importorskip("torch")
    scenes = W.uneven_batch(9, seed=21, min_side=17, max_side=131, min_tri=20, max_tri=1500, tex_size=32,
                            use_vbo=False)
    want = plain(gpu, scenes)
    ctxs, streams = setup_frames(gpu, scenes)
    launches = {}
    for mode in (1, 0):
        b = gpu.batch(tile_size=16, readback_kernel=mode)
        for _ in range(2):
            keep, hosts = [], []
            for i, s in enumerate(scenes):
                n = s.width * s.height
                if i % 3 == 2:  # pageable
                    hosts.append(np.zeros((s.height, s.width), np.uint32))
                    continue
                off = 1 if i % 3 == 1 else 0  # one word past a 16-byte boundary
                t = torch.zeros(n + 4, dtype=torch.int32, pin_memory=True)
                keep.append(t)
                hosts.append(t.numpy().view(np.uint32)[off:off + n].reshape(s.height, s.width))
            gpu.play_many(ctxs, streams)
            b.reset_stats()
            b.render(ctxs, colors=hosts)
            b.wait()
            launches[mode] = b.stats()["kernel_launches"]
            for h, w, s in zip(hosts, want, scenes):
                assert np.array_equal(h, w[0]), f"{s.name} (readback_kernel={mode})"
        b.destroy()
    assert launches[1] == launches[0] + 1
    for c in ctxs:
        c.destroy()


@pytest.mark.slow
def test_full_uneven_batch_matches_oracle(gpu, oracle):
    """All 256 frames of the benchmark's uneven batch (sides 64-1024, 100-200k triangles, seed
    3) rendered by one mtgl_batch_render with the tuned defaults, each against the oracle
    rendering the same frame alone: depth and stencil exact, colour within 1 LSB."""
    scenes = W.uneven_batch(256)
    ctxs, streams = setup_frames(gpu, scenes)
    b = gpu.batch()
    for _ in range(2):  # the second run replays the captured graph
        gpu.play_many(ctxs, streams)
        b.render(ctxs)
    b.wait()
    got = read_all(ctxs)
    b.destroy()
    for c in ctxs:
        c.destroy()

    def check(i):
        s = scenes[i]
        stats = harness.compare(render(oracle, s), got[i], harness.cleared_buffers(s))
        harness.assert_parity(stats, color_tol=1, name=s.name)
        return stats["color_max_err"]

    order = sorted(range(len(scenes)), key=lambda i: -W.scene_triangles(scenes[i]))
    with cf.ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        errs = list(ex.map(check, order))
    assert len(errs) == 256 and max(errs) <= 1
