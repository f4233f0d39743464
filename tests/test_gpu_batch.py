"""Multi-scene batches (lucent_batch_*): several renderers traced as one
wavefront must give, bit for bit, what each renderer gives traced alone
(same random streams, same kernels, same per-pixel accumulation order),
whatever the wave size, with or without the captured CUDA graph, and mixed
with single-renderer traces."""
import numpy as np
import pytest

from lucent_gb300 import workloads as W
from lucent_gb300._native import LucentError
from lucent_gb300.renderer import Batch, Renderer

pytestmark = pytest.mark.gpu


def _specs():
    """(scene, width, height, max bounces): the batched workload's generator
    at small sizes, the box scene, and the knot scene with dielectrics and
    alpha-blended triangles."""
    out = []
    for seed in range(3):
        sc, _ = W.batch_scene(seed, tri_lo=2_000, tri_hi=20_000)
        out.append((sc, 48 + 16 * seed, 40, 6))
    out.append((W.box_scene(1, 3), 64, 48, 8))
    out.append((W.knot_scene(0, tubular=200, radial=16, env_width=256), 40, 40, 12))
    return out


@pytest.fixture(scope="module")
def specs():
    return _specs()


def _renderers(specs):
    rs = []
    for i, (sc, w, h, mb) in enumerate(specs):
        r = Renderer(w, h)
        r.settings.max_bounces = mb
        r.load_scene(sc)
        r.set_seed(100 * i)
        rs.append(r)
    return rs


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


@pytest.fixture(scope="module")
def solo(specs):
    rs = _renderers(specs)
    for r in rs:
        r.trace_samples(5)
    out = [r.read() for r in rs]
    for r in rs:
        r.dispose()
    return out


@pytest.mark.parametrize("opts", [{}, {"samples_per_wave": 2}, {"samples_per_wave": 1, "use_graph": False},
                                  {"max_wave_paths": 5000}, {"samples_per_wave": 3},
                                  {"sort_rays": False, "top_levels": False}, {"wide_bvh": False},
                                  {"scenes_per_wave": 1}, {"scenes_per_wave": 2, "samples_per_wave": 2},
                                  {"scenes_per_wave": 2, "use_graph": False, "max_wave_paths": 5000},
                                  {"streams": 2}, {"streams": 3, "scenes_per_wave": 1, "samples_per_wave": 2}])
def test_batch_equals_renderers_alone(specs, solo, opts):
    rs = _renderers(specs)
    b = Batch(rs, **opts)
    b.trace_samples(3)
    b.trace_samples(2)
    st = b.check()
    assert st["closest_rays"] > 0 and st["shadow_rays"] > 0
    if opts.get("use_graph", True) and st["waves"] > 2:
        assert st["graph_waves"] > 0
    for r, ref in zip(rs, solo):
        got = r.read()
        assert not np.isnan(got[0]).any()
        assert np.all(got[3] == 5)
        assert _same(got, ref)
    b.dispose()
    for r in rs:
        r.dispose()


def test_batch_beyond_the_staged_top_levels(specs):
    # Shared memory holds the top BVH levels of the first 8 scenes; the rays
    # of later scenes read every node from global memory.
    specs10 = (specs * 2)[:10]
    rs = _renderers(specs10)
    for r in rs:
        r.trace_samples(2)
    ref = [r.read() for r in rs]
    for r in rs:
        r.dispose()
    rs = _renderers(specs10)
    b = Batch(rs)
    b.trace_samples(2)
    b.check()
    for r, want in zip(rs, ref):
        assert _same(r.read(), want)
    b.dispose()
    for r in rs:
        r.dispose()


def test_batch_mixed_with_single_traces(specs, solo):
    rs = _renderers(specs)
    b = Batch(rs, samples_per_wave=1)
    b.trace_samples(2)
    rs[1].trace_samples(3)  # one renderer alone in between
    b2 = Batch([r for i, r in enumerate(rs) if i != 1])
    b2.trace_samples(3)
    b2.check()
    for r, ref in zip(rs, solo):
        assert _same(r.read(), ref)
    for x in (b, b2, *rs):
        x.dispose()


def test_batch_errors(specs):
    sc, w, h, mb = specs[0]
    r = Renderer(w, h)
    r.load_scene(sc)
    with pytest.raises(LucentError):
        Batch([r, r])
    empty = Renderer(8, 8)  # no scene loaded
    b = Batch([r, empty])
    with pytest.raises(LucentError):
        b.trace_samples(1)
    with pytest.raises(LucentError):
        b.set_options(max_wave_paths=0)
    for bad in (0, 17):
        with pytest.raises(LucentError):
            b.set_options(max_wave_paths=1 << 20, streams=bad)
    b.set_options(streams=2)  # a part without a scene fails as the whole batch does
    with pytest.raises(LucentError):
        b.trace_samples(1)
    for x in (b, r, empty):
        x.dispose()


def test_autotuned_batch_equals_renderers_alone(specs, solo):
    # Whatever the autotuner picks (wave size, graph replay, ray sorting, top
    # levels, grid sizes), the images are those of the renderers alone.
    rs = _renderers(specs)
    b = Batch(rs)
    opts, times = b.autotune(samples=1)
    assert len(times) >= 2 and set(opts) >= {"sort_rays", "top_levels", "shade_blocks"}
    for i, r in enumerate(rs):
        r.reset()
        r.set_seed(100 * i)
    b.trace_samples(5)
    b.check()
    for r, ref in zip(rs, solo):
        assert _same(r.read(), ref)
    b.dispose()
    for r in rs:
        r.dispose()
