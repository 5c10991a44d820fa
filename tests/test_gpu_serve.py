"""The serving loop (mtgl_serve.h) on the GPU: requests admitted against a memory budget,
batched on several executors, rendered into pooled framebuffers and read back.

Each request's colour must match the CPU oracle rendering the same calls on a context of
the request's size (within 1 LSB), and must be bit-identical whether the request is
served alone or in a loaded mix (the alone-vs-mix test).
"""
import numpy as np
import pytest

import harness
from mytinygl_gb300 import gl as G
from mytinygl_gb300 import workloads as W

pytestmark = pytest.mark.gpu

RES = ((32, 32), (64, 64), (100, 60), (128, 96))


@pytest.fixture(scope="module")
def gpu():
    return harness.product()


@pytest.fixture(scope="module")
def oracle():
    return harness.oracle()


@pytest.fixture(scope="module")
def scenes():
    return W.serve_scenes(4, seed=21, min_tri=200, max_tri=3000, tex_sizes=(32, 64), width=128, height=96)


def make_server(gpu, scenes, **kw):
    srv = gpu.server(**kw)
    ctxs = []
    for sc in scenes:
        c = gpu.context(sc.width, sc.height)
        k = W.frame_start(sc)
        sc.play(c, 0, k)
        c.glFinish()
        ctxs.append(c)
        srv.add_scene(c, sc.stream(k), W.scene_triangles(sc))
    return srv, ctxs


def requests(trace):
    reqs = (G.Request * len(trace))()
    outs = []
    for i, (t, sc, w, h, mv) in enumerate(trace):
        out = np.zeros((h, w), np.uint32)
        outs.append(out)
        reqs[i].scene, reqs[i].width, reqs[i].height = sc, w, h
        reqs[i].modelview[:] = [float(v) for v in mv]
        reqs[i].color = out.ctypes.data
        reqs[i].arrival = t
    return reqs, outs


def oracle_frame(oracle, scene, w, h, mv):
    ctx = oracle.context(w, h)
    k = W.frame_start(scene)
    scene.play(ctx, 0, k)
    ctx.glViewport(0, 0, w, h)
    ctx.glMatrixMode(G.GL_MODELVIEW)
    ctx.glLoadMatrixf(np.asarray(mv, np.float32))
    scene.play(ctx, k)
    c, _, _ = ctx.read(depth=False, stencil=False)
    ctx.destroy()
    return c


def serve(gpu, scenes, trace, **kw):
    srv, ctxs = make_server(gpu, scenes, **kw)
    reqs, outs = requests(trace)
    base = srv.now() + 0.01
    for r in reqs:
        r.arrival += base
    srv.run_trace(reqs)
    stats = srv.stats()
    srv.destroy()
    for c in ctxs:
        c.destroy()
    return reqs, outs, stats


def test_served_frames_match_oracle(gpu, oracle, scenes):
    trace = W.serve_trace(0.02, 2000.0, nscenes=len(scenes), seed=22, resolutions=RES)
    reqs, outs, stats = serve(gpu, scenes, trace, executors=2, max_batch=8)
    assert stats["completed"] == len(trace) and stats["failed"] == 0, stats
    assert stats["batches"] >= 2
    for r, out, (t, sc, w, h, mv) in zip(reqs, outs, trace):
        assert r.status == 0 and r.finished >= r.admitted >= r.arrival > 0
        want = oracle_frame(oracle, scenes[sc], w, h, mv)
        d = np.abs(want.view(np.uint8).astype(np.int16) - out.view(np.uint8).astype(np.int16))
        assert d.max() <= 1, (sc, w, h, int(d.max()))


def test_alone_equals_in_the_mix(gpu, scenes):
    """Every request of a loaded trace, served again alone, gives the same frame bit for bit."""
    trace = W.serve_trace(0.03, 3000.0, nscenes=len(scenes), seed=23, resolutions=RES)
    _, mixed, _ = serve(gpu, scenes, trace, executors=3, max_batch=6)
    srv, ctxs = make_server(gpu, scenes)
    for i, (t, sc, w, h, mv) in enumerate(trace):
        reqs, alone = requests([(0.0, sc, w, h, mv)])
        reqs[0].arrival = srv.now()
        srv.run_trace(reqs)
        assert reqs[0].status == 0
        assert np.array_equal(alone[0], mixed[i]), i
    srv.destroy()
    for c in ctxs:
        c.destroy()


@pytest.mark.slow
def test_served_sample_of_the_benchmark_scenes(gpu, oracle):
    """A seeded sample of requests from the serving benchmark's own trace (32 resident scenes
    of 1k-500k triangles with 256^2-2048^2 textures, resolutions up to 1920x1080), served in
    one burst, against the oracle rendering the same calls."""
    import concurrent.futures as cf
    import os

    scenes = W.serve_scenes(32)
    trace = W.serve_trace(60.0, 2000.0, seed=6)
    pick = sorted(np.random.default_rng(62).choice(len(trace), size=12, replace=False))
    sample = [(0.0,) + tuple(trace[int(i)][1:]) for i in pick]
    reqs, outs, stats = serve(gpu, scenes, sample, executors=2, max_batch=64)
    assert stats["completed"] == len(sample) and stats["failed"] == 0, stats

    def check(i):
        _, sc, w, h, mv = sample[i]
        want = oracle_frame(oracle, scenes[sc], w, h, mv)
        d = np.abs(want.view(np.uint8).astype(np.int16) - outs[i].view(np.uint8).astype(np.int16))
        assert d.max() <= 1, (sc, w, h, int(d.max()))

    order = sorted(range(len(sample)), key=lambda i: -W.scene_triangles(scenes[sample[i][1]]))
    with cf.ThreadPoolExecutor(os.cpu_count() or 1) as ex:
        list(ex.map(check, order))


def request_cost(gpu, scene, w, h):
    """The server's admission cost of a request (framebuffer + pipeline-scratch estimate)."""
    cfg = G.BatchConfig()
    gpu.lib.mtgl_dev_batch_defaults(cfg)
    per_tri = 3 * 48 + 8 + cfg.record_factor * (244 + cfg.pair_factor * 16)
    return w * h * 9 + int(per_tri * W.scene_triangles(scene))


def test_budget_defers_and_refuses(gpu, scenes):
    trace = [(0.0, sc, w, h, mv) for _, sc, w, h, mv in
             W.serve_trace(0.01, 4000.0, nscenes=len(scenes), seed=24, resolutions=RES)]
    _, full, _ = serve(gpu, scenes, trace)
    # all queued at once, room for the largest request alone: everything still completes
    one = max(request_cost(gpu, scenes[sc], w, h) for _, sc, w, h, _ in trace)
    _, tight, st = serve(gpu, scenes, trace, memory_budget=one, executors=2, max_batch=4)
    assert st["completed"] == len(trace) and st["deferred_for_budget"] > 0, st
    for a, b in zip(full, tight):
        assert np.array_equal(a, b)
    # a request larger than the whole budget, and one naming no scene, fail alone
    bad = [(0.0, 0, 4096, 4096, trace[0][4]), (0.0, 99, 32, 32, trace[0][4]), (0.0, 1, 32, 32, trace[0][4])]
    reqs, _, st = serve(gpu, scenes, bad, memory_budget=64 << 20)
    assert [r.status for r in reqs] == [7, 1, 0]  # MTGL_ERR_OVERFLOW, MTGL_ERR_INVALID, served
