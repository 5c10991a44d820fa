"""The oracle is pinned: bit-exact against the reference's own output (CPU only).

1. golden fixtures rendered by the reference build (tests/golden, regenerated by
   tests/golden/make_golden.py) — these travel with the repository;
2. where the reference sources exist, the reference build itself on the feature scenes,
   on seeded random scenes and on the headline workloads.
"""
import numpy as np
import pytest

import feature_scenes as F
import harness
from mytinygl_gb300 import workloads as W
from mytinygl_gb300.scene import render


@pytest.fixture(scope="module")
def oracle():
    return harness.oracle()


@pytest.fixture(scope="module")
def ref():
    r = harness.reference()
    if r is None:
        pytest.skip("reference sources not present")
    return r


@pytest.mark.parametrize("path", harness.golden_files(), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_oracle_matches_golden(oracle, path):
    scene, expected, buffers = harness.load_golden(path)
    got = render(oracle, scene)
    stats = harness.compare(expected, got, buffers)
    harness.assert_parity(stats, color_tol=0, name=scene.name)


@pytest.mark.parametrize("name", sorted(F.SCENES))
def test_oracle_matches_reference_feature(oracle, ref, name):
    scene = F.SCENES[name][0]()
    stats = harness.compare(render(ref, scene), render(oracle, scene), harness.cleared_buffers(scene))
    harness.assert_parity(stats, color_tol=0, name=name)


@pytest.mark.parametrize("seed", range(6))
def test_oracle_matches_reference_random(oracle, ref, seed):
    """Random mixes of state, primitives and geometry."""
    rng = np.random.default_rng(100 + seed)
    s = F.base(f"random{seed}", 80, 60)
    modes = [F.G.GL_TRIANGLES, F.G.GL_TRIANGLE_STRIP, F.G.GL_TRIANGLE_FAN, F.G.GL_QUADS, F.G.GL_POLYGON]
    for _ in range(6):
        if rng.random() < 0.5:
            s.glEnable(F.G.GL_DEPTH_TEST)
        else:
            s.glDisable(F.G.GL_DEPTH_TEST)
        if rng.random() < 0.4:
            s.glEnable(F.G.GL_BLEND)
            s.glBlendFunc(F.G.GL_SRC_ALPHA, F.G.GL_ONE_MINUS_SRC_ALPHA)
        else:
            s.glDisable(F.G.GL_BLEND)
        s.glShadeModel([F.G.GL_SMOOTH, F.G.GL_FLAT][int(rng.integers(0, 2))])
        F.rand_tris(s, rng, int(rng.integers(2, 8)), spread=float(rng.uniform(1, 6)), z=(-12.0, 2.0),
                    alpha=(0.0, 1.0), mode=modes[int(rng.integers(0, len(modes)))])
    stats = harness.compare(render(ref, s), render(oracle, s))
    harness.assert_parity(stats, color_tol=0, name=s.name)


@pytest.mark.parametrize("which", ["sphere", "sphere_client", "textured", "rop"])
def test_oracle_matches_reference_headline(oracle, ref, which):
    scene = {
        "sphere": lambda: W.sphere_scene(),
        "sphere_client": lambda: W.sphere_scene(use_vbo=False, seed=5),
        "textured": lambda: W.textured_scene(480, 270, ntri=4000),
        "rop": lambda: W.rop_scene(480, 270, ntri=40000),
    }[which]()
    stats = harness.compare(render(ref, scene), render(oracle, scene), harness.cleared_buffers(scene))
    harness.assert_parity(stats, color_tol=0, name=which)


SIZE_CASES = [((16384, 1), True), ((1, 16384), True), ((16385, 1), False), ((1, 16385), False), ((0, 4), False),
              ((4, 0), False), ((-1, 4), False)]


def context_created(lib, w, h):
    h_ = lib.lib.gl_create_context(w, h)
    if h_:
        lib.lib.gl_destroy_context(h_)
    return bool(h_)


def test_context_size_limits(oracle):
    """Framebuffer sides are 1..16384 (framebuffer.h:30-35): larger or empty ones are refused."""
    for (w, h), ok in SIZE_CASES:
        assert context_created(oracle, w, h) == ok, (w, h)


def test_context_size_limits_match_reference(ref):
    for (w, h), ok in SIZE_CASES:
        assert context_created(ref, w, h) == ok, (w, h)
