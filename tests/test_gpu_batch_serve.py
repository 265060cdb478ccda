"""Batched scenes and the continuous-batching server on the GPU."""
import numpy as np
import pytest

from gpu_util import torch_cuda
from oracle import ref

pytestmark = pytest.mark.gpu


def _small_config3(count=12, seed=3):
    from sphgb import scenes
    return scenes.config3_specs(n_scenes=count, seed=seed, n_min=1024, n_max=8192)


def test_batched_equals_plain_and_matches_oracle_density():
    """The batched path (all scenes in one graph launch) and the plain path
    (one scene per launch) give bit-identical states; the density of the first
    step is within 1e-4 of the FP64 oracle for every scene."""
    torch_cuda()
    from sphgb.batch import run_batched, run_plain
    pairs = _small_config3()
    _, one = run_batched(pairs, 1)
    for (spec, st), got in zip(pairs, one):
        sp = ref.params_from_spec(spec)
        _, _, rho = ref.step(sp, st.position, st.velocity)
        assert np.max(np.abs(got.density - rho) / rho) < 1e-4
    tb, sb = run_batched(pairs, 6)
    tp, sp_ = run_plain(pairs, 6)
    tg, sg = run_plain(pairs, 6, use_graph=True)
    for a, b, c in zip(sb, sp_, sg):
        for f in ("position", "velocity", "density"):
            np.testing.assert_array_equal(getattr(a, f), getattr(b, f))
            np.testing.assert_array_equal(getattr(a, f), getattr(c, f))
    assert tb > 0 and tp > 0 and tg > 0


def _requests(count, seed, rate):
    from sphgb import scenes
    from sphgb.serve import poisson_requests

    def make(rng):
        spec, st, steps = scenes.served_request(rng, n_min=1024, n_max=16384)
        return spec, st, int(rng.integers(3, 25))
    return poisson_requests(rate, count, seed=seed, make=make)


def test_server_results_identical_alone_and_in_the_mix():
    """Requests served with continuous batching (arrivals while others run,
    admission under a tight HBM budget, re-packing as scenes come and go)
    give exactly the state each scene reaches when run alone."""
    torch_cuda()
    from sphgb.device import SceneBatch
    from sphgb.serve import SceneServer, footprint
    reqs = _requests(10, seed=4, rate=400.0)
    budget = 2.5 * max(footprint(r.spec) for r in reqs)     # forces queueing
    server = SceneServer(hbm_budget_bytes=budget, max_tick_steps=8)
    stats = server.run(reqs)
    server.close()
    assert stats.requests == 10 and len(stats.latencies) == 10
    assert stats.repacks >= 2 and stats.ticks >= 3
    assert np.isfinite(stats.pct(50)) and stats.pct(99) >= stats.pct(50)
    for r in reqs:
        alone = SceneBatch([r.spec])
        alone.load_states([r.state])
        alone.step(r.steps)
        a = alone.states()[0]
        alone.close()
        for f in ("position", "velocity", "density"):
            np.testing.assert_array_equal(getattr(r.result, f), getattr(a, f),
                                          err_msg=f"request {r.rid} ({r.spec.mode}) {f}")


def test_server_refuses_a_request_over_budget():
    torch_cuda()
    from sphgb.serve import SceneServer, footprint
    reqs = _requests(1, seed=5, rate=1000.0)
    server = SceneServer(hbm_budget_bytes=footprint(reqs[0].spec) - 1)
    with pytest.raises(MemoryError):
        server.run(reqs)
    server.close()


def test_reconfigure_and_tuning_keep_results():
    """Re-packing a context and changing launch tuning leave results unchanged."""
    torch_cuda()
    from sphgb import _capi, scenes
    from sphgb.device import SceneBatch
    spec, st = scenes.config0()
    base = SceneBatch([spec])
    base.load_states([st])
    base.step(3)
    want = base.states()[0]
    other, ost = scenes.pipe_flow(n=5000, seed=2, h=0.05)
    b = SceneBatch([other])
    b.reconfigure([spec])                  # smaller scratch needs: buffers reused
    for tuning in ((128, _capi.DENSITY_THREAD, 16), (512, _capi.DENSITY_WARP, 256)):
        b.set_tuning(*tuning)
        b.load_states([st])
        b.step(3)
        got = b.states()[0]
        for f in ("position", "velocity", "density"):
            np.testing.assert_array_equal(getattr(got, f), getattr(want, f), err_msg=str(tuning))
    b.close()
    base.close()


def test_batched_workload_every_scene_against_the_oracle():
    """The batched workload at its full size (256 boxes, 1,024-65,536
    particles each, one context): after one batched step, every scene's
    neighbour rows and counts equal the FP64 oracle's capped lists bit for
    bit, and its density is within 1e-5 (relative, per particle; the
    small-case bound); its first step's conservation sums equal FP64 sums of
    its own state."""
    torch_cuda()
    from sphgb import scenes
    from sphgb.device import SceneBatch
    from test_gpu_full_size import _lists_without_self
    pairs = scenes.config3_specs(n_scenes=256, seed=3)
    b = SceneBatch([p[0] for p in pairs])
    b.load_states([p[1] for p in pairs])
    b.step(1)
    got = b.states()
    lst, cnt = (t.cpu().numpy() for t in b.step_neighbours())
    cons = b.conservation()
    b.close()
    worst = 0.0
    for k, ((spec, st), g) in enumerate(zip(pairs, got)):
        off = b.scene_offsets[k]
        sp = ref.params_from_spec(spec)
        spid, start, count = ref.organize(sp, ref.assign_voxels(sp, st.position))
        want_l, _, _ = ref.neighbours(sp, st.position, spid, start, count)
        rows, kk = _lists_without_self(want_l)
        np.testing.assert_array_equal(cnt[off:off + spec.n], kk, err_msg=f"scene {k}")
        np.testing.assert_array_equal(lst[off:off + spec.n], rows, err_msg=f"scene {k}")
        rho = ref.density(sp, st.position, spid, start, count)
        err = float(np.max(np.abs(g.density - rho) / rho))
        worst = max(worst, err)
        assert err < 1e-5, (k, err)
        m = np.float64(np.float32(spec.constants.mass))
        assert abs(cons[k][0] - m * spec.n) <= 1e-12 * m * spec.n
        assert cons[k][7] == spec.n
    print(f"256 scenes: density max rel err {worst:.1e}")
