"""Batched and served forms (pt_render_batch, pt_autotune, pt_server_*).

A path's sample streams depend only on its own job (seed, pixel, sample
index), so a job rendered in a batch, or a request served among others, gives
the same film as the job rendered alone: bit for bit when the per-pixel
summation is grouped the same way, otherwise within FP32 summation rounding
(relative 1e-5).
"""
from __future__ import annotations

import numpy as np
import pytest

from pathtracer_gb300 import native as N
from pathtracer_gb300 import scene as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes(renderer):
    cb, cam_cb = S.cornell_icosphere(3)
    rg, cam_rg = S.rough_glass(subdiv=3, env_w=128, env_h=64, seed=2)
    md, cam_md = S.material_divergence(subdiv=2, seed=3, aspect=1.0)
    ids = [renderer.upload(cb), renderer.upload(rg), renderer.upload(md)]
    yield list(zip(ids, [cam_cb, cam_rg, cam_md]))
    for sid in ids:
        renderer.release(sid)


def _jobs(scenes):
    (s0, c0), (s1, c1), (s2, c2) = scenes
    return [
        N.job_desc(s0, c0, 48, 40, 4, 2, 8, seed=1, estimator=N.EST_NEE_MIS),
        N.job_desc(s1, c1, 32, 32, 2, 2, 12, seed=2, estimator=N.EST_NEE_MIS, env_sampling=N.ENV_ALIAS,
                   rr_start=4),
        N.job_desc(s2, c2, 40, 24, 4, 4, 6, seed=3, estimator=N.EST_NEE_MIS, sampler=N.SAMPLER_STRATIFIED),
        N.job_desc(s0, c0, 16, 16, 8, 8, 8, seed=4, estimator=N.EST_REF_NEE),
    ]


def test_batch_matches_individual(renderer, scenes):
    jobs = _jobs(scenes)
    films, st = renderer.render_batch(jobs, stats=True)
    assert st.paths == sum(j.width * j.height * j.spp_x * j.spp_y for j in jobs)
    for j, f in zip(jobs, films):
        alone = renderer.render(j)
        assert np.isfinite(f).all()
        assert np.allclose(f, alone, rtol=1e-5, atol=1e-7), np.abs(f - alone).max()


def test_batch_graph_replay_identical(renderer, scenes):
    jobs = _jobs(scenes)
    a = renderer.render_batch(jobs)
    b = renderer.render_batch(jobs)  # replay of the captured graph
    c = renderer.render_batch(jobs[::-1])[::-1]  # another composition
    for x, y, z in zip(a, b, c):
        assert np.array_equal(x, y)
        assert np.array_equal(x, z)


def test_batch_empty_and_invalid(renderer, scenes):
    assert renderer.render_batch([]) == []
    bad = _jobs(scenes)[:1]
    bad[0].scene = 999
    with pytest.raises(N.PtError):
        renderer.render_batch(bad)


def test_autotune_picks_a_candidate(scenes):
    # a context of its own: the tuned launch configuration stays with it
    r = N.Renderer(0)
    cb, cam_cb = S.cornell_icosphere(3)
    md, cam_md = S.material_divergence(subdiv=2, seed=3, aspect=1.0)
    a, b = r.upload(cb), r.upload(md)
    jobs = [N.job_desc(a, cam_cb, 64, 48, 4, 4, 8, seed=1, estimator=N.EST_NEE_MIS),
            N.job_desc(b, cam_md, 32, 32, 2, 4, 6, seed=3, estimator=N.EST_NEE_MIS,
                       sampler=N.SAMPLER_STRATIFIED)]
    renderer = r
    ref = renderer.render_batch(jobs)
    t = renderer.autotune(jobs)
    assert t["candidates"] == 24
    assert t["wave_paths"] in (1 << 20, 1 << 22, 1 << 24)
    assert t["sort_by_material"] in (0, 1)
    assert 0.0 < t["best_ms"] <= t["default_ms"] + 1e-9
    after = renderer.render_batch(jobs)
    # the tuned configuration may shade through the generic kernel instead of
    # the per-family ones (separately compiled arithmetic, so a rare path can
    # branch differently): the images agree statistically, nearly all pixels
    # to rounding
    for x, y in zip(ref, after):
        close = np.isclose(x, y, rtol=1e-4, atol=1e-6).all(-1)
        assert close.mean() > 0.95, close.mean()
        assert abs(float(x.mean()) - float(y.mean())) <= 2e-2 * float(x.mean())
    r.close()


def test_batch_persistent_equals_graph(renderer, scenes):
    """PT_BATCH_PERSISTENT (one cooperative launch per scene group, all waves
    and bounces, grid barriers between the stages) renders the same samples
    as the per-stage graph form: the same path / vertex / ray counts and the
    same films up to FP32 rounding of the generically compiled shading (the
    graph form shades per material family), across several waves."""
    jobs = _jobs(scenes)
    films_g, st_g = renderer.render_batch(jobs, stats=True)
    renderer.set_batch_mode(N.BATCH_PERSISTENT)
    try:
        films_p, st_p = renderer.render_batch(jobs, stats=True)
        again = renderer.render_batch(jobs)
    finally:
        renderer.set_batch_mode(N.BATCH_GRAPH)
    assert st_p.paths == st_g.paths
    for a, b, c in zip(films_p, films_g, again):
        assert np.isfinite(a).all()
        assert np.array_equal(a, c)  # deterministic
        close = np.isclose(a, b, rtol=1e-4, atol=1e-6).all(-1)
        assert close.mean() > 0.99, close.mean()
    with pytest.raises(N.PtError):
        renderer.set_batch_mode(7)


def test_batch_persistent_many_waves(monkeypatch):
    # tiny waves: the persistent kernel loops over many waves of each group
    monkeypatch.setenv("PT_WAVE_PATHS", "4096")
    small = N.Renderer(0)
    try:
        sc, cam = S.cornell_icosphere(2)
        sid = small.upload(sc)
        job = N.job_desc(sid, cam, 32, 24, 4, 4, 6, seed=9, estimator=N.EST_NEE_MIS)
        ref = small.render(job)
        small.set_batch_mode(N.BATCH_PERSISTENT)
        films = small.render_batch([job, job])
        for f in films:
            assert np.isclose(f, ref, rtol=1e-4, atol=1e-6).all(-1).mean() > 0.99
    finally:
        small.close()


def _serve_until_done(srv, ids, max_steps=10000):
    for _ in range(max_steps):
        if srv.step() == 0:
            break
    out = {}
    for rid in ids:
        st, film, spp, lat = srv.poll(rid)
        assert st == N.REQ_DONE, st
        assert lat >= 0.0
        out[rid] = (film, spp)
    return out


def test_served_same_alone_and_in_mix(renderer, scenes):
    jobs = _jobs(scenes)
    probe = jobs[0]
    # alone
    srv = N.Server(renderer, hbm_budget=1 << 30, max_slots=8)
    rid = srv.submit(probe, spp_per_pass=2)
    alone, spp_alone = _serve_until_done(srv, [rid])[rid]
    srv.close()
    assert spp_alone == probe.spp_x * probe.spp_y
    # in a mix: one request already running, others arriving mid-flight
    srv = N.Server(renderer, hbm_budget=1 << 30, max_slots=8)
    first = srv.submit(jobs[1], spp_per_pass=1)
    srv.step()
    rid = srv.submit(probe, spp_per_pass=2)
    srv.step()
    late = [srv.submit(jobs[2], spp_per_pass=4), srv.submit(jobs[3], spp_per_pass=8)]
    res = _serve_until_done(srv, [first, rid] + late)
    srv.close()
    mixed, spp_mixed = res[rid]
    assert spp_mixed == spp_alone
    assert np.array_equal(alone, mixed)
    # and the served film is the job's film (pass sums grouped differently)
    ref = renderer.render(probe)
    assert np.allclose(mixed, ref, rtol=1e-5, atol=1e-7)
    for r, j in zip([first] + late, [jobs[1], jobs[2], jobs[3]]):
        assert np.allclose(res[r][0], renderer.render(j), rtol=1e-5, atol=1e-7)


def test_served_rmse_target_and_cap(renderer, scenes):
    jobs = _jobs(scenes)
    srv = N.Server(renderer, hbm_budget=1 << 30, max_slots=4)
    easy = srv.submit(jobs[0], target_rmse=1e9, spp_per_pass=1)  # met once both halves have a pass
    capped = srv.submit(jobs[3], spp_cap=6, spp_per_pass=4)
    res = _serve_until_done(srv, [easy, capped])
    srv.close()
    assert res[easy][1] == 2
    assert res[capped][1] == 6


def test_served_paths_per_pass(renderer, scenes):
    """paths_per_pass sizes each pass from the request's own pixels (never
    below spp_per_pass): the same result alone and in a mix, and the job's
    film up to FP32 grouping."""
    jobs = _jobs(scenes)
    probe = jobs[1]
    px = probe.width * probe.height
    srv = N.Server(renderer, hbm_budget=1 << 30, max_slots=8)
    rid = srv.submit(probe, spp_per_pass=1, paths_per_pass=3 * px)  # 3 spp per pass
    alone, spp_alone = _serve_until_done(srv, [rid])[rid]
    srv.close()
    srv = N.Server(renderer, hbm_budget=1 << 30, max_slots=8)
    other = srv.submit(jobs[2], spp_per_pass=2, paths_per_pass=1)  # floor: 2 spp per pass
    srv.step()
    rid = srv.submit(probe, spp_per_pass=1, paths_per_pass=3 * px)
    res = _serve_until_done(srv, [other, rid])
    srv.close()
    assert res[rid][1] == spp_alone == probe.spp_x * probe.spp_y
    assert np.array_equal(alone, res[rid][0])
    assert np.allclose(alone, renderer.render(probe), rtol=1e-5, atol=1e-7)
    assert np.allclose(res[other][0], renderer.render(jobs[2]), rtol=1e-5, atol=1e-7)
    srv = N.Server(renderer, hbm_budget=1 << 30, max_slots=8)
    with pytest.raises(N.PtError):
        srv.submit(probe, spp_per_pass=1, paths_per_pass=-5)
    srv.close()


def test_served_srpt_small_first_same_results(renderer, scenes):
    """Shortest remaining work first: with a pass budget below the large
    request's work, the small requests finish before it; every result equals
    the same request served alone (a request's samples depend on its own job
    only); a full queue refuses with PT_ERR_BUSY; queueing delay and latency
    are reported."""
    jobs = _jobs(scenes)
    big, small = jobs[3], [jobs[0], jobs[1], jobs[2]]
    alone = {}
    for k, j in enumerate([big] + small):
        srv = N.Server(renderer, hbm_budget=1 << 30, max_slots=8)
        rid = srv.submit(j, spp_per_pass=2)
        alone[k] = _serve_until_done(srv, [rid])[rid]
        srv.close()
    srv = N.Server(renderer, hbm_budget=1 << 30, max_slots=8)
    budget = min(j.width * j.height * 2 for j in small)
    srv.set_policy(N.SERVE_SRPT, pass_paths=budget, max_queue=4)
    ids = [srv.submit(big, spp_per_pass=2)] + [srv.submit(j, spp_per_pass=2) for j in small]
    with pytest.raises(N.PtError) as ei:
        srv.submit(small[0], spp_per_pass=2)  # four requests wait: the queue is full
    assert ei.value.code == -6
    done_order = []
    while len(done_order) < len(ids):
        srv.step()
        for rid in ids:
            if rid not in done_order and srv.poll(rid)[0] == N.REQ_DONE:
                done_order.append(rid)
    assert done_order[-1] == ids[0]  # the large request finishes last
    for k, rid in enumerate(ids):
        st, film, spp, lat = srv.poll(rid)
        assert np.array_equal(film, alone[k][0]) and spp == alone[k][1]
        q, lat2 = srv.times(rid)
        assert 0.0 <= q <= lat2
    srv.close()


def test_server_admission_by_budget_and_cancel(renderer, scenes):
    jobs = _jobs(scenes)
    j = jobs[0]
    film_bytes = 2 * j.width * j.height * 3 * 4
    srv = N.Server(renderer, hbm_budget=film_bytes, max_slots=8)  # one request's films at a time
    a = srv.submit(j, spp_per_pass=8)
    b = srv.submit(j, spp_per_pass=8)
    c = srv.submit(j, spp_per_pass=8)
    srv.cancel(c)
    srv.step()
    st_b = srv.poll(b)[0]
    assert st_b == N.REQ_QUEUED  # no room until a's films are released
    res = _serve_until_done(srv, [a, b])
    assert srv.poll(c)[0] == N.REQ_CANCELLED
    srv.close()
    assert np.array_equal(res[a][0], res[b][0])


def test_multi_wave_render_equals_single_wave(renderer, scenes, monkeypatch):
    # a context with a tiny wave capacity renders the job in many waves that
    # overlap on two queue sets; films add samples in sample order, so the
    # result has the single-wave bits
    monkeypatch.setenv("PT_WAVE_PATHS", "4096")
    small = N.Renderer(0)
    monkeypatch.delenv("PT_WAVE_PATHS")
    cb, cam = S.cornell_icosphere(3)
    md, cam_md = S.material_divergence(subdiv=2, seed=3, aspect=1.0)
    for sc, c, kw in ((cb, cam, {}), (md, cam_md, {"sampler": N.SAMPLER_STRATIFIED})):
        a_id, b_id = renderer.upload(sc), small.upload(sc)
        ja = N.job_desc(a_id, c, 40, 36, 4, 2, 6, seed=8, estimator=N.EST_NEE_MIS, **kw)
        jb = N.job_desc(b_id, c, 40, 36, 4, 2, 6, seed=8, estimator=N.EST_NEE_MIS, **kw)
        one, st1 = renderer.render(ja, stats=True)
        many, st2 = small.render(jb, stats=True)
        assert st1.paths == st2.paths == 40 * 36 * 8
        assert st1.rays == st2.rays and st1.shadow_rays == st2.shadow_rays
        assert np.array_equal(one, many)
        renderer.release(a_id)
        small.release(b_id)
    small.close()


def test_paired_tracing_equals_separate_tracing(renderer, scenes, monkeypatch):
    # small waves trace bounce b's shadow rays with bounce b + 1's closest
    # rays in one launch; the shadow terms are still added before the next
    # shade pass, so the film has the bits of separate launches
    monkeypatch.setenv("PT_PAIR_TRACE", "0")
    sep = N.Renderer(0)
    monkeypatch.delenv("PT_PAIR_TRACE")
    for sc, c, kw in ((S.cornell_icosphere(3)[0], S.cornell_icosphere(3)[1], {}),
                      (*S.material_divergence(subdiv=2, seed=3, aspect=1.0), {"sampler": N.SAMPLER_STRATIFIED}),
                      (*S.rough_glass(subdiv=4, env_w=256, env_h=128, seed=2),
                       {"rr_start": 4, "env_sampling": N.ENV_ALIAS})):
        a_id, b_id = renderer.upload(sc), sep.upload(sc)
        ja = N.job_desc(a_id, c, 48, 40, 4, 4, 8, seed=6, estimator=N.EST_NEE_MIS, **kw)
        jb = N.job_desc(b_id, c, 48, 40, 4, 4, 8, seed=6, estimator=N.EST_NEE_MIS, **kw)
        paired, st1 = renderer.render(ja, stats=True)
        separate, st2 = sep.render(jb, stats=True)
        assert st1.rays == st2.rays and st1.shadow_rays == st2.shadow_rays
        assert np.array_equal(paired, separate)
        renderer.release(a_id)
        sep.release(b_id)
    sep.close()


def test_traversal_cap_reports_device_error_and_context_survives(monkeypatch):
    # failure detection without a fault: a context whose traversal step bound
    # is tiny makes every ray hit it; the kernels set the device error flag
    # and return, the call reports PT_ERR_DEVICE, and the context (and the
    # GPU) stay usable
    monkeypatch.setenv("PT_TRAVERSAL_CAP", "2")
    r = N.Renderer(0)
    monkeypatch.delenv("PT_TRAVERSAL_CAP")
    sc, cam = S.cornell_icosphere(2)
    sid = r.upload(sc)
    job = N.job_desc(sid, cam, 16, 16, 1, 1, 4)
    with pytest.raises(N.PtError) as e:
        r.render(job)
    assert e.value.code == -5
    with pytest.raises(N.PtError):
        r.render_batch([job])
    v = r.sampler_eval(N.SAMPLER_HALTON_NONE, 1, 4, 2)  # the context still works
    assert np.allclose(v[:, 0], [0.5, 0.25, 0.75, 0.125])
    r.release(sid)
    r.close()
    ok = N.Renderer(0)  # and so does a fresh one
    sid = ok.upload(sc)
    assert np.isfinite(ok.render(N.job_desc(sid, cam, 16, 16, 1, 1, 4))).all()
    ok.release(sid)
    ok.close()
