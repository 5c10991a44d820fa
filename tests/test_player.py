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
