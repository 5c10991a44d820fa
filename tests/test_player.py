"""The native command-stream player (mtgl_play) on the CPU oracle: a stream replays a scene
exactly like the per-call binding, and the generated player matches include/GL/gl.h."""
import numpy as np

import feature_scenes as F
import harness
from mytinygl_gb300 import gen_play
from mytinygl_gb300.scene import render


def test_generated_player_is_current():
    with open(gen_play.OUT) as f:
        assert f.read() == gen_play.generate(), "run python -m mytinygl_gb300.gen_play"


def test_player_function_ids_match_library():
    lib = harness.oracle()
    assert lib.lib.mtgl_play_function_count() == len(gen_play.FUNCTIONS) == 111


def test_stream_replays_scenes_like_calls():
    lib = harness.oracle()
    for name in ("blend", "stencil", "texture_modes", "display_lists", "vbo", "draw_pixels", "lighting_phong"):
        s = F.SCENES[name][0]()
        want = render(lib, s)
        ctx = lib.context(s.width, s.height)
        lib.play(ctx, s.stream())
        c, d, st = ctx.read()
        got = (c, d, st, ctx.glGetError())
        ctx.destroy()
        stats = harness.compare(want, got, harness.cleared_buffers(s))
        assert stats["color_max_err"] == 0 and stats["depth_mismatches"] == 0 and stats["stencil_mismatches"] == 0
        assert stats["error_equal"], name


def test_malformed_stream_is_refused():
    lib = harness.oracle()
    ctx = lib.context(8, 8)
    bad = np.array([9999, 0], np.uint32).tobytes()
    assert lib.lib.mtgl_play(ctx.handle, bad, len(bad)) != 0
    short = np.array([gen_play.FUNCTION_ID["glClear"], 1], np.uint32).tobytes()  # argument slot missing
    assert lib.lib.mtgl_play(ctx.handle, short, len(short)) != 0
    ctx.destroy()


def _play_all(lib, scenes, threads, monkeypatch, dup=False):
    monkeypatch.setenv("MTGL_PLAY_THREADS", str(threads))
    ctxs = [lib.context(s.width, s.height) for s in scenes]
    streams = [s.stream() for s in scenes]
    if dup:  # the first context twice: its two streams must play in order, on one thread
        ctxs.append(ctxs[0])
        streams.append(scenes[0].stream())
    lib.play_many(ctxs, streams)
    out = [(*c.read(), c.glGetError()) for c in ctxs[:len(scenes)]]
    for c in ctxs[:len(scenes)]:
        c.destroy()
    return out


def test_play_many_threads_match_serial(monkeypatch):
    """Contexts played concurrently render exactly what one thread renders, with the same
    errors; a list naming a context twice falls back to one thread and keeps call order."""
    lib = harness.oracle()
    names = ("blend", "stencil", "texture_modes", "list_blocks", "vbo", "draw_pixels", "lighting_phong", "fog",
             "vertex_arrays", "extreme_values", "clip_big", "lines_states")
    scenes = [F.SCENES[n][0]() for n in names]
    serial = _play_all(lib, scenes, 1, monkeypatch)
    for threads, dup in ((4, False), (16, False), (4, True)):
        got = _play_all(lib, scenes, threads, monkeypatch, dup)
        for name, s, a, b in zip(names, scenes, serial, got):
            if dup and s is scenes[0]:
                continue  # played twice
            stats = harness.compare(a, b, harness.cleared_buffers(s))
            assert stats["color_max_err"] == 0 and stats["depth_mismatches"] == 0, (name, threads)
            assert stats["stencil_mismatches"] == 0 and stats["error_equal"], (name, threads)


def test_play_many_reports_first_failure(monkeypatch):
    """Every stream plays; the status is the lowest-index failure's."""
    lib = harness.oracle()
    monkeypatch.setenv("MTGL_PLAY_THREADS", "3")
    s = F.SCENES["blend"][0]()
    ctxs = [lib.context(s.width, s.height) for _ in range(3)]
    bad = np.array([9999, 0], np.uint32).tobytes()
    with np.testing.assert_raises(RuntimeError):
        lib.play_many(ctxs, [bad, s.stream(), s.stream()])
    c0 = ctxs[1].read()[0]
    c1 = ctxs[2].read()[0]
    assert (c0 == c1).all() and c0.any()
    for c in ctxs:
        c.destroy()
