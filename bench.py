"""Benchmark of the wavefront path integrator (one JSON line on rank 0).

Workload (default): the rough-glass scene -- a seeded displaced icosphere of
1,310,720 triangles (subdivision 8, radial noise 0.05) in rough glass (ior
1.5, alpha 0.05) over a GGX conductor ground (alpha 0.2), lit by a seeded
1024x512 FP32 HDRI (sky gradient + 3 Gaussian sun lobes, peak 5e3), rendered
at 1024x1024, 256 spp (16x16 grid), depth 16, Russian roulette from depth 4,
Owen-scrambled Halton sampler.  The estimator is the drop-in's: REF_NEE
(getRayColor of maxdepth_nee.hpp restated: 4 light samples per vertex,
uniform-sphere environment sampling), the estimator the CPU arm runs, so the
GPU/CPU ratio compares one algorithm.  ``nee_mis`` reports the same steps
with NEE+MIS and the luminance alias table beside it, with its own CPU
figure from the oracle's iterative NEE+MIS.
One step = 16 of the 256 samples per pixel for every pixel (16.8 M paths,
one wave), so every kernel launch of the timed region runs alone and its
CUDA-event duration is the kernel's (the roofline).  ``per_call`` reports
the same job rendered 32 spp per call (two waves that overlap on two queue
sets), how a full frame is rendered in practice.

  value  paths/s with the scene resident in HBM, device film, device time
         (CUDA events on the library's stream, max over ranks);
  e2e    the same metric through the public C-ABI call pt_render with a
         pinned HOST film: the job descriptor and offset table go host->device
         and the 12.6 MB film device->host inside every step.
  roofline  the dominant stage (traversal) as the contract's single kernel
         figure, and under ``stages`` every queue stage's algorithmic bytes
         (unit costs in STAGE_UNIT_BYTES) over its CUDA-event time.

``--impl reference`` times the reference algorithm on the host cores: the
CPU restatement of the reference integrator (oracle/pt_oracle.cpp, REF_NEE,
all hardware threads) on a bounded sample of the same workload.

Multi-GPU (torchrun): the path is sample-parallel, every rank renders its own
sample range of the same frame (replicas, no collective on the data path);
``value`` = all ranks' paths / max-over-ranks time (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

import numpy as np  # noqa: E402

PEAKS = REPO / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
# ncu DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of all
# traversal-stage launches (closest, paired, shadow and the shadow resolve) of
# one step of 16 spp of every pixel, per (workload, estimator); from a
# one-pass ncu capture of the same bench command
NCU_TRAVERSAL_BYTES_PER_STEP = {("rough_glass", 0): 8.850e9}
# Algorithmic queue bytes per unit, by stage: the records each stage must
# read or write in this layout -- 192 B per path vertex,
# 88 B per shadow ray (44 written by shade, 44 read by the traversal) and FP32
# film; each byte charged to the stage that moves it:
#   camera    64 B per path: ray origin + direction (32) and path state
#             (throughput + pdf 16, radiance 16) written
#   traversal 48 B per closest-hit ray: ray read (32) + hit written (16);
#             44 B per shadow ray: ShadowQueue record read
#   sort      16 B per closest-hit ray: key + index written and read (8 x 2)
#   shade     128 B per path vertex: hit read (16) + path state read and written (80)
#             + continuation RayQueue record written (32);
#             44 B per shadow ray: ShadowQueue record written
#   film      16 B per path: its radiance read; 24 B per film pixel per wave:
#             FP32 RGB read-modify-write
STAGE_UNIT_BYTES = {"camera": {"paths": 64}, "traversal": {"rays": 48, "shadow_rays": 44},
                    "sort": {"rays": 16}, "shade": {"segments": 128, "shadow_rays": 44},
                    "film": {"paths": 16, "film_pixel_waves": 24}}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="rough_glass", choices=["rough_glass", "cornell", "divergence"])
    ap.add_argument("--estimator", default="ref_nee", choices=["ref_nee", "nee_mis"],
                    help="ref_nee: the drop-in's estimator (also the CPU arm's); nee_mis: NEE+MIS + alias env")
    ap.add_argument("--spp-per-step", type=int, default=16)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched and served forms")
    ap.add_argument("--no-rmse", action="store_true", help="skip the converged-reference RMSE")
    ap.add_argument("--batch-jobs", type=int, default=96)
    ap.add_argument("--serve-seconds", type=float, default=10.0)
    ap.add_argument("--serve-rate", type=float, default=20.0, help="Poisson arrivals per second")
    ap.add_argument("--serve-pass-spp", type=int, default=16, help="samples per request per scheduling pass")
    ap.add_argument("--serve-pass-paths", type=int, default=1 << 21,
                    help="paths per request per scheduling pass (0: pass-spp only)")
    ap.add_argument("--config4-seconds", type=float, default=120.0,
                    help="arrival window of the served config-4 mix (20 req/s; 0: skip)")
    ap.add_argument("--config4-drain", type=float, default=20.0,
                    help="seconds the config-4 server keeps running after the arrivals end")
    ap.add_argument("--persistent-config3", action="store_true",
                    help="also time the config-3 batch in the persistent form (about two more minutes)")
    return ap.parse_args()


WORKLOADS = {
    # name: (width, height, spp_x, spp_y, depth, rr_start, estimator, sampler, env_sampling, description)
    "rough_glass": dict(W=1024, H=1024, sx=16, sy=16, depth=16, rr=4, est=0, sampler=2, env=0,
                        desc="rough-glass displaced icosphere (1,310,720 tris) + conductor ground + "
                             "1024x512 HDRI, 1024x1024, 256 spp, depth 16, RR from 4"),
    "cornell": dict(W=256, H=256, sx=8, sy=8, depth=8, rr=-1, est=0, sampler=2, env=0,
                    desc="Cornell box + 5120-tri GGX gold icosphere, 256x256, 64 spp, depth 8"),
    "divergence": dict(W=1920, H=1080, sx=16, sy=8, depth=12, rr=-1, est=0, sampler=3, env=0,
                       desc="64 icospheres x 20480 tris, 5 material families, homogeneous medium, "
                            "1920x1080, 128 spp, depth 12, stratified"),
}


ESTIMATORS = {"ref_nee": dict(est=0, env=0, name="REF_NEE (maxdepth_nee.hpp restated), uniform-sphere env sampling"),
              "nee_mis": dict(est=1, env=1, name="NEE+MIS (power heuristic), luminance alias-table env sampling")}


def workload(name: str, estimator: str) -> dict:
    """The workload's settings with the estimator's (est, env) fields."""
    wl = dict(WORKLOADS[name])
    e = ESTIMATORS[estimator]
    wl.update(est=e["est"], env=e["env"], est_name=e["name"])
    return wl


def sample_chunk(step: int, rank: int, world: int, n_chunks: int) -> int:
    """Replica sharding: at each step every rank takes its own chunk of the
    frame's sample grid (disjoint across ranks within a step; steps cycle
    through the grid)."""
    return (step * world + rank) % n_chunks


def max_over_ranks(value: float, dist: bool, device=None) -> float:
    """Max of a per-rank timing over all ranks (torch.distributed)."""
    if not dist:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def build_scene(name):
    from pathtracer_gb300 import scene as S

    if name == "rough_glass":
        return S.rough_glass(8)
    if name == "cornell":
        return S.cornell_icosphere(4)
    return S.material_divergence(5)


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = max(mx, float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def stage_roofline(prof: dict, tot: dict, peak: float) -> dict:
    """Per queue stage: algorithmic bytes (STAGE_UNIT_BYTES x the stage's unit
    counts over the timed steps), CUDA-event milliseconds, GB/s and the
    fraction of the HBM peak.  traversal = the trace and shadow stages
    (closest, paired and shadow launches + resolve)."""
    counts = {"paths": tot["paths"], "segments": tot["segments"], "rays": tot["rays"], "shadow_rays": tot["shadow"],
              "film_pixel_waves": tot["film_pixel_waves"]}
    ms = {"camera": prof["camera"][0], "traversal": prof["trace"][0] + prof["shadow"][0], "sort": prof["sort"][0],
          "shade": prof["shade"][0], "film": prof["film"][0]}
    out = {}
    for st, units in STAGE_UNIT_BYTES.items():
        b = float(sum(u * counts[c] for c, u in units.items()))
        gbs = b / (ms[st] / 1e3) / 1e9 if ms[st] > 0 else None
        out[st] = {"bytes": b, "ms": ms[st], "achieved_gbs": gbs, "frac": gbs / peak if gbs else None,
                   "unit_bytes": units}
    return out


def cpu_paths_per_sec(osc, cam, wl, estimator, threads, target_s=12.0, max_px=1024):
    """Times the CPU restatement of the reference integrator on a bounded
    sample (a square crop-free frame of up to max_px^2 pixels at 1 spp of
    the workload's sample grid), sized to about target_s of CPU work."""
    from pathtracer_gb300 import native as N

    res = 64
    # calibrate the sample size to about target_s of CPU work
    while True:
        job = N.job_desc(0, cam, res, res, wl["sx"], wl["sy"], wl["depth"], estimator=estimator,
                         sampler=wl["sampler"], rr_start=wl["rr"], env_sampling=0 if estimator == 0 else wl["env"],
                         seed=7, spp_begin=0, spp_end=1)
        t0 = time.perf_counter()
        osc.render(job, threads=threads)
        dt = time.perf_counter() - t0
        if dt > target_s / 4 or res >= max_px:
            break
        res = min(max_px, int(res * max(1.5, min(4.0, (target_s / 4 / max(dt, 1e-3)) ** 0.5))))
    t0 = time.perf_counter()
    osc.render(job, threads=threads)
    dt = time.perf_counter() - t0
    return res * res / dt, f"{res}x{res} pixels x 1 spp of the workload's scene and camera", dt


def run_full_frames(r, names, cpu: bool, threads: int) -> dict:
    """The other single-job workloads (configs 0 and 2) at their full size:
    one whole frame (every sample) per estimator through pt_render with a
    host film -- device time from the library's events, e2e from the wall
    clock around the call -- and, with `cpu`, the oracle's REF_NEE on a
    bounded sample of the same scene on the host cores."""
    from pathtracer_gb300 import native as N

    out = {}
    for name in names:
        sc, cam = build_scene(name)
        sid = r.upload(sc)
        res = {"workload": WORKLOADS[name]["desc"]}
        for est in ("ref_nee", "nee_mis"):
            wl = workload(name, est)
            job = N.job_desc(sid, cam, wl["W"], wl["H"], wl["sx"], wl["sy"], wl["depth"], rr_start=wl["rr"],
                             estimator=wl["est"], sampler=wl["sampler"], env_sampling=wl["env"], seed=1)
            warm = N.job_desc(sid, cam, wl["W"], wl["H"], wl["sx"], wl["sy"], wl["depth"], rr_start=wl["rr"],
                              estimator=wl["est"], sampler=wl["sampler"], env_sampling=wl["env"], seed=1,
                              spp_begin=0, spp_end=1)
            r.render(warm)
            t0 = time.perf_counter()
            film, st = r.render(job, stats=True)
            wall = time.perf_counter() - t0
            res[est] = {"paths": int(st.paths), "paths_per_s": st.paths / (st.ms / 1e3),
                        "e2e_paths_per_s": st.paths / wall, "rays_per_s": (st.rays + st.shadow_rays) / (st.ms / 1e3),
                        "frame_s": wall, "finite": bool(np.isfinite(film).all()), "estimator": wl["est_name"]}
        if cpu:
            from oracle import pyoracle as O

            wl = workload(name, "ref_nee")
            v, sample, dt = cpu_paths_per_sec(O.OracleScene(sc), cam, wl, wl["est"], threads, target_s=6.0)
            res["cpu_baseline"] = {"value": v, "unit": "paths/s", "cores": threads, "kind": "port",
                                   "sample": sample + f" ({dt:.1f} s), REF_NEE"}
            res["e2e_vs_cpu"] = res["ref_nee"]["e2e_paths_per_s"] / v
        r.release(sid)
        out[name] = res
    return out


def form_scenes(r, with_big: bool):
    """The resident scenes of the batched and served forms: the three
    workloads with seeded per-object motion (meshes and spheres move, walls,
    ground and area lights stay), plus for serving the 5,242,880-triangle
    displaced-sphere variant of the rough-glass scene.  Values: (scene id,
    camera, focus distance)."""
    from pathtracer_gb300 import native as N
    from pathtracer_gb300 import scene as S

    out = {}
    t0 = time.perf_counter()
    sc, cam = S.cornell_icosphere(4)
    out["cornell"] = (r.upload(S.with_motion(sc, seed=21)), cam, 1.9)
    sc, cam = S.rough_glass(8)
    out["rough_glass"] = (r.upload(S.with_motion(sc, seed=22)), cam, 4.24)
    sc, cam = S.material_divergence(5)
    out["divergence"] = (r.upload(S.with_motion(sc, seed=23)), cam, 11.9)
    big = None
    upload_s = {}
    if with_big:
        sc, cam = S.rough_glass(9, seed=5)
        sc = S.with_motion(sc, seed=24)
        # time to first pixel of the big scene: upload (BVH build, items,
        # copies) with the reference's trees and with SAH trees on the host,
        # then with the device mesh builder, which the served form keeps
        for key, b in (("reference_tree_host", N.BVH_BUILD_HOST), ("sah_host", N.BVH_BUILD_SAH)):
            r.set_bvh_builder(b)
            t1 = time.perf_counter()
            r.release(r.upload(sc))
            upload_s[key] = round(time.perf_counter() - t1, 3)
        r.set_bvh_builder(N.BVH_BUILD_DEVICE)
        t1 = time.perf_counter()
        big = (r.upload(sc), cam, 4.24)
        upload_s["device_builder"] = round(time.perf_counter() - t1, 3)
        r.set_bvh_builder(N.BVH_BUILD_HOST)
    return out, big, time.perf_counter() - t0, upload_s


def run_batched(r, scenes, n_jobs: int, seed: int = 11, res=(64, 1024), spp=(4, 256), tune: bool = True,
                tune_sample: int = 8, tune_spp: int = 4, persistent: bool = True):
    """Config-3 job mix: one pt_render_batch call (one CUDA-graph launch)
    against the plain wavefront drop-in (pt_render per job, one after the
    other); both with host films, so both are end to end.  The two arms
    render the same samples, so their images (and RMSE) are equal; the
    largest relative film difference is reported."""
    from pathtracer_gb300 import scene as S

    jobs = S.job_mix(scenes, n_jobs, seed=seed, res=res, spp=spp)
    paths = sum(j.width * j.height * j.spp_x * j.spp_y for j in jobs)
    tuning, tune_s = None, 0.0
    if tune:
        # autotune the batch launch on a sample of the mix (the first jobs,
        # their spp capped at tune_spp)
        tj = []
        for j in jobs[:tune_sample]:
            jj = type(j).from_buffer_copy(j)
            if jj.spp_x * jj.spp_y > tune_spp:
                jj.spp_begin, jj.spp_end = 0, tune_spp
            tj.append(jj)
        t0 = time.perf_counter()
        tuning = r.autotune(tj)
        tune_s = time.perf_counter() - t0
    # warm: queue allocation and graph capture
    r.render_batch(jobs)
    t0 = time.perf_counter()
    films_b, st = r.render_batch(jobs, stats=True)
    t_batch = time.perf_counter() - t0
    pers = None
    if persistent:
        # the same batch as ONE persistent cooperative launch per scene group
        from pathtracer_gb300 import native as N
        r.set_batch_mode(N.BATCH_PERSISTENT)
        try:
            r.render_batch(jobs)
            t0 = time.perf_counter()
            films_q, st_q = r.render_batch(jobs, stats=True)
            t_pers = time.perf_counter() - t0
        finally:
            r.set_batch_mode(N.BATCH_GRAPH)
        rel_q = 0.0
        for a, b in zip(films_q, films_b):
            rel_q = max(rel_q, float(np.abs(a - b).max() / max(1e-12, float(np.abs(b).max()))))
    # plain wavefront, one job after the other (warm the context's queues first)
    r.render(jobs[0])
    t0 = time.perf_counter()
    films_p = [r.render(j) for j in jobs]
    t_plain = time.perf_counter() - t0
    rel = 0.0
    for a, b in zip(films_b, films_p):
        d = np.abs(a - b).max() / max(1e-12, float(np.abs(b).max()))
        rel = max(rel, float(d))
    if persistent:
        pers = {"paths_per_s": paths / t_pers, "speedup_vs_plain": t_plain / t_pers, "vs_graph": t_batch / t_pers,
                "device_ms": st_q.ms, "max_rel_film_diff_vs_graph": rel_q,
                "form": "one cooperative launch per scene group: every wave and bounce, grid barriers between "
                        "stages, generic (unsorted) shading"}
    sides = sorted(j.width for j in jobs)
    out = {
        "jobs": n_jobs, "paths": paths, "paths_per_s": paths / t_batch, "plain_paths_per_s": paths / t_plain,
        "speedup_vs_plain": t_plain / t_batch, "batch_s": t_batch, "plain_s": t_plain,
        "graph_device_ms": st.ms, "max_rel_film_diff_vs_plain": rel,
        "equal_rmse": "same samples in both arms: identical images up to FP32 summation order",
        "mix": f"{n_jobs} jobs over cornell/rough_glass/divergence with per-object motion; square resolution "
               f"log-uniform {res[0]}..{res[1]} (median {sides[len(sides) // 2]}), spp U{{{spp[0]}..{spp[1]}}}, "
               "lens diameter U[0,0.05], shutter U[0,0.5], NEE+MIS",
        "autotune": ({k: tuning[k] for k in ("wave_paths", "sort_by_material", "trace_blocks", "shade_blocks")} |
                     {"candidates": tuning["candidates"], "seconds": tune_s}) if tuning else "as tuned above",
    }
    if pers is not None:
        out["persistent"] = pers
    return out


def run_served(r, scenes, big, seconds: float, rate: float, seed: int = 12, pass_spp: int = 8,
               pass_paths: int = 0):
    """Serving: Poisson arrivals at `rate` req/s for `seconds` over the
    resident scenes; each request a seeded camera, square resolution
    log-uniform 128..512, an spp cap U{16..128} and a target RMSE of 0.02
    (whichever comes first), `pass_spp` spp per scheduling pass.  Latency is from the
    request's arrival to its completion.  The plain arm renders the same
    requests (same samples, spp as served) one after the other through
    pt_render."""
    from pathtracer_gb300 import native as N
    from pathtracer_gb300 import scene as S

    rng = np.random.default_rng(seed)
    pool = dict(scenes)
    if big is not None:
        pool["rough_glass_5m"] = big
    names = sorted(pool)
    reqs = []
    t = 0.0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t > seconds:
            break
        name = names[int(rng.integers(len(names)))]
        key = "rough_glass" if name == "rough_glass_5m" else name
        sid, cam, focus = pool[name]
        side = int(round(np.exp(rng.uniform(np.log(128), np.log(512)))))
        cap = int(rng.integers(16, 129))
        job = S.job_mix({key: (sid, cam, focus)}, 1, seed=int(rng.integers(1 << 30)), res=(side, side),
                        spp=(cap, cap))[0]
        reqs.append((t, job, cap))
    srv = N.Server(r, hbm_budget=32 << 30, max_slots=64)
    lat, spp_done = {}, {}
    arrival = {}
    outstanding = set()
    busy = 0.0
    k = 0
    t0 = time.perf_counter()
    while k < len(reqs) or outstanding:
        now = time.perf_counter() - t0
        while k < len(reqs) and reqs[k][0] <= now:
            rid = srv.submit(reqs[k][1], target_rmse=0.02, spp_cap=reqs[k][2], spp_per_pass=pass_spp,
                             paths_per_pass=pass_paths)
            arrival[rid] = (reqs[k][0], k)
            outstanding.add(rid)
            k += 1
        if not outstanding:
            time.sleep(max(0.0, reqs[k][0] - (time.perf_counter() - t0)))
            continue
        s0 = time.perf_counter()
        srv.step()
        busy += time.perf_counter() - s0
        now = time.perf_counter() - t0
        for rid in list(outstanding):
            st, n = srv.state(rid)
            if st >= N.REQ_DONE:
                outstanding.discard(rid)
                lat[rid] = (now - arrival[rid][0]) * 1e3
                spp_done[arrival[rid][1]] = n
    wall = time.perf_counter() - t0
    srv.close()
    served_paths = sum(reqs[i][1].width * reqs[i][1].height * n for i, n in spp_done.items())
    # plain arm: the same requests at the spp they were served with
    t0 = time.perf_counter()
    for i, n in spp_done.items():
        j = reqs[i][1]
        j.spp_begin, j.spp_end = 0, n
        r.render(j)
    t_plain = time.perf_counter() - t0
    ls = sorted(lat.values())
    pct = lambda q: ls[min(len(ls) - 1, int(q * len(ls)))] if ls else None
    return {
        "requests": len(reqs), "completed": len(lat), "rate_req_s": rate, "seconds": seconds,
        "p50_ms": pct(0.50), "p99_ms": pct(0.99), "max_ms": ls[-1] if ls else None,
        "paths": served_paths, "paths_per_s_busy": served_paths / busy if busy else None,
        "paths_per_s_wall": served_paths / wall, "plain_paths_per_s": served_paths / t_plain,
        "speedup_vs_plain": t_plain / busy if busy else None,
        "mean_spp": float(np.mean(list(spp_done.values()))) if spp_done else None,
        "mix": "4 resident scenes (cornell, rough_glass 1.3M tris, divergence, rough_glass 5.2M tris) with motion; "
               f"res log-uniform 128..512, spp cap U{{16..128}}, target RMSE 0.02, {pass_spp} spp per pass"
               + (f" (or ~{pass_paths} paths per request per pass)" if pass_paths else ""),
    }


def run_served_config4(r, scenes, big, seconds: float, rate: float, drain: float, seed: int = 14,
                       pass_paths: int = 1 << 27, max_queue: int = 512, max_slots: int = 256,
                       request_pass_paths: int = 1 << 22):
    """The served workload as specified for serving: Poisson arrivals at
    `rate` req/s for `seconds` over the 4 resident scenes (Cornell, rough glass
    1.3 M tris, material divergence, rough glass 5.2 M tris), each request a
    seeded camera, square resolution log-uniform 128..2048, an spp cap
    U{16..1024} and a target RMSE of 0.02 (whichever first).  Admission by
    free HBM and slots, SRPT scheduling (pt_server_set_policy: the least
    remaining work first, `pass_paths` per pass; each request's chunk per pass
    is enough samples for about `request_pass_paths` paths, at least 16 spp),
    a bounded queue (PT_ERR_BUSY
    beyond `max_queue` waiting requests: refused).  The loop runs until the
    arrivals end plus `drain` seconds; requests still unfinished then are
    cancelled and counted.  This mix asks for far more paths than one GPU
    renders in that time (a 2048^2 request at its cap is 4.3 G paths), so the
    numbers describe an overloaded server: which requests finish, and how
    fast."""
    from pathtracer_gb300 import native as N
    from pathtracer_gb300 import scene as S

    rng = np.random.default_rng(seed)
    pool = dict(scenes)
    if big is not None:
        pool["rough_glass_5m"] = big
    names = sorted(pool)
    reqs = []
    t = 0.0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t > seconds:
            break
        name = names[int(rng.integers(len(names)))]
        key = "rough_glass" if name == "rough_glass_5m" else name
        sid, cam, focus = pool[name]
        side = int(round(np.exp(rng.uniform(np.log(128), np.log(2048)))))
        cap = int(rng.integers(16, 1025))
        job = S.job_mix({key: (sid, cam, focus)}, 1, seed=int(rng.integers(1 << 30)), res=(side, side),
                        spp=(cap, cap))[0]
        reqs.append((t, job, cap, side))
    srv = N.Server(r, hbm_budget=64 << 30, max_slots=max_slots)
    srv.set_policy(N.SERVE_SRPT, pass_paths=pass_paths, max_queue=max_queue)
    refused, outstanding, ids = 0, set(), {}
    done = {}
    busy, k, passes = 0.0, 0, 0
    t0 = time.perf_counter()
    while True:
        now = time.perf_counter() - t0
        while k < len(reqs) and reqs[k][0] <= now:
            try:
                rid = srv.submit(reqs[k][1], target_rmse=0.02, spp_cap=reqs[k][2], spp_per_pass=16,
                                 paths_per_pass=request_pass_paths)
                ids[rid] = k
                outstanding.add(rid)
            except N.PtError as e:
                if e.code != -6:
                    raise
                refused += 1
            k += 1
        if now > seconds + drain:
            break
        if not outstanding:
            if k >= len(reqs):
                break
            time.sleep(max(0.0, min(reqs[k][0], seconds + drain) - (time.perf_counter() - t0)))
            continue
        s0 = time.perf_counter()
        srv.step()
        busy += time.perf_counter() - s0
        passes += 1
        for rid in list(outstanding):
            st, n = srv.state(rid)
            if st >= N.REQ_DONE:
                outstanding.discard(rid)
                if st == N.REQ_DONE:
                    done[rid] = n
    wall = time.perf_counter() - t0
    queued_at_end = sum(1 for rid in outstanding if srv.state(rid)[0] == N.REQ_QUEUED)
    lat, qd = [], []
    for rid in ids:
        q, l_ms = srv.times(rid)
        if q >= 0:
            qd.append(q)
        if rid in done:
            lat.append(l_ms)
    for rid in outstanding:
        srv.cancel(rid)
    srv.close()
    paths = sum(reqs[ids[rid]][1].width * reqs[ids[rid]][1].height * n for rid, n in done.items())
    lat.sort()
    qd.sort()
    pct = lambda v, q: v[min(len(v) - 1, int(q * len(v)))] if v else None
    sides = [reqs[ids[rid]][3] for rid in done]
    return {
        "rate_req_s": rate, "arrival_seconds": seconds, "drain_seconds": drain, "arrivals": len(reqs),
        "submitted": len(ids), "refused_queue_full": refused, "completed": len(done),
        "unfinished_cancelled": len(outstanding), "still_queued_at_end": queued_at_end,
        "p50_ms": pct(lat, 0.5), "p99_ms": pct(lat, 0.99), "max_ms": lat[-1] if lat else None,
        "queue_delay_p50_ms": pct(qd, 0.5), "queue_delay_p99_ms": pct(qd, 0.99),
        "completed_median_side": int(np.median(sides)) if sides else None,
        "completed_max_side": max(sides) if sides else None,
        "mean_spp_completed": float(np.mean(list(done.values()))) if done else None,
        "paths_completed": paths, "paths_per_s_busy": paths / busy if busy else None,
        "passes": passes, "wall_s": wall,
        "mix": "4 resident scenes (cornell, rough_glass 1.3M tris, divergence, rough_glass 5.2M tris) with "
               "motion; res log-uniform 128..2048, spp cap U{16..1024}, target RMSE 0.02, NEE+MIS; SRPT "
               f"with {pass_paths} paths per pass, ~{request_pass_paths} paths (>= 16 spp) per request per pass, "
               f"queue bound {max_queue}, {max_slots} slots",
    }


def converged_rmse(r, sid, cam, wl, k_step: int, win: int = 64, ref_grid: int = 256):
    """RMSE of the workload's render against a converged reference on the
    frame's centre window: the reference is the GPU render of that window at
    ref_grid^2 = 65536 spp (a window job has the full frame's sample
    streams; the GPU against the oracle at high spp on small windows is
    tests/test_gpu_converged.py).  Reported for one bench step (k_step spp)
    and for the workload's full spp."""
    from pathtracer_gb300 import native as N

    W, H = wl["W"], wl["H"]
    x0, y0 = (W - win) // 2, (H - win) // 2

    def job(sx, sy, begin=0, end=0, seed=1):
        j = N.job_desc(sid, cam, win, win, sx, sy, wl["depth"], rr_start=wl["rr"], estimator=wl["est"],
                       sampler=wl["sampler"], env_sampling=wl["env"], seed=seed, spp_begin=begin, spp_end=end)
        j.crop_x, j.crop_y, j.full_width, j.full_height = x0, y0, W, H
        return j

    t0 = time.perf_counter()
    ref = r.render(job(ref_grid, ref_grid, seed=977))
    ref_s = time.perf_counter() - t0
    full = r.render(job(wl["sx"], wl["sy"]))
    step = r.render(job(wl["sx"], wl["sy"], 0, k_step))
    rm = lambda a: float(np.sqrt(np.mean((a.astype(np.float64) - ref) ** 2)))
    return {"reference": f"GPU {ref_grid * ref_grid} spp on the {win}x{win} centre window of the "
                         f"{W}x{H} frame (independent seed); oracle spot-check in tests/test_gpu_converged.py",
            "rmse_full_spp": rm(full), "full_spp": wl["sx"] * wl["sy"], "rmse_step_spp": rm(step),
            "step_spp": k_step, "reference_seconds": ref_s,
            "equal_rmse_forms": "batched and served jobs render the same samples as the plain path"}


def run_reference(args, rank, world):
    wl = workload(args.workload, args.estimator)
    if rank != 0:
        return
    from oracle import pyoracle as O

    sc, cam = build_scene(args.workload)
    osc = O.OracleScene(sc)
    threads = os.cpu_count() or 1
    vals, secs = [], []
    sample = ""
    for i in range(args.warmup + args.steps):
        v, sample, dt = cpu_paths_per_sec(osc, cam, wl, wl["est"], threads,
                                          target_s=max(4.0, 90.0 / (args.steps + args.warmup)))
        if i >= args.warmup:
            vals.append(v)
            secs.append(dt)
    value = statistics.median(vals)
    line = {
        "impl": "reference", "metric": "paths/s", "value": value, "unit": "paths/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(secs),
        "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
        "config": {"workload": wl["desc"], "estimator": wl["est_name"]},
        "cpu_baseline": {"value": value, "unit": "paths/s", "cores": threads, "kind": "port",
                         "sample": sample + "; oracle/pt_oracle.cpp, the CPU restatement of the reference path"},
        "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, local_rank):
    import torch

    from pathtracer_gb300 import native as N

    wl = workload(args.workload, args.estimator)
    torch.cuda.set_device(local_rank)
    r = N.Renderer(local_rank)
    sc, cam = build_scene(args.workload)
    sid = r.upload(sc)
    info = r.scene_info(sid)
    W, H = wl["W"], wl["H"]
    spp_total = wl["sx"] * wl["sy"]
    k = args.spp_per_step

    def job_for(step, scene_id=None):
        chunk = sample_chunk(step, rank, world, max(1, spp_total // k))
        return N.job_desc(sid if scene_id is None else scene_id, cam, W, H, wl["sx"], wl["sy"], wl["depth"],
                          rr_start=wl["rr"],
                          estimator=wl["est"], sampler=wl["sampler"], env_sampling=wl["env"], seed=1,
                          spp_begin=chunk * k, spp_end=chunk * k + k)

    film = torch.zeros(H * W * 3, dtype=torch.float32, device=f"cuda:{local_rank}")
    dist = world > 1

    def barrier():
        torch.cuda.synchronize()
        if dist:
            torch.distributed.barrier()

    # ---- device-resident timing (value)
    for i in range(args.warmup):
        r.render_device(job_for(i), film.data_ptr(), sync=True)
    barrier()
    r.profile_begin()
    stats = N.Stats()
    tot = dict(paths=0, segments=0, rays=0, shadow=0, bytes=0, film_pixel_waves=0)
    t_dev = 0.0
    with ClockSampler(local_rank) as clk:
        barrier()
        w0 = time.perf_counter()
        for i in range(args.steps):
            st = r.render_device(job_for(args.warmup + i), film.data_ptr(), sync=False, stats=True)
            t_dev += st.ms
            tot["paths"] += st.paths
            tot["segments"] += st.segments
            tot["rays"] += st.rays
            tot["shadow"] += st.shadow_rays
            tot["bytes"] += st.algorithmic_bytes
            tot["film_pixel_waves"] += W * H  # one wave per step
        barrier()
        wall = time.perf_counter() - w0
    prof = r.profile_end()
    del stats
    t_max = t_dev / 1e3
    paths_all = tot["paths"]
    if dist:
        tt = torch.tensor([t_max], device=f"cuda:{local_rank}", dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_max = float(tt.item())
        pt = torch.tensor([paths_all], device=f"cuda:{local_rank}", dtype=torch.float64)
        torch.distributed.all_reduce(pt)
        paths_all = int(pt.item())
    value = paths_all / t_max

    # ---- end-to-end through pt_render with a pinned host film
    host = torch.empty((H, W, 3), dtype=torch.float32, pin_memory=True)
    hp = host.numpy()
    lib = N.load()
    e2e_steps = max(2, args.steps // 2)
    job = job_for(0)
    lib.pt_render(r.ctx, C.byref(job), hp.ctypes.data_as(C.POINTER(C.c_float)), None)
    barrier()
    e0 = time.perf_counter()
    e2e_paths = 0
    for i in range(e2e_steps):
        job = job_for(args.warmup + i)
        rc = lib.pt_render(r.ctx, C.byref(job), hp.ctypes.data_as(C.POINTER(C.c_float)), None)
        if rc != 0:
            raise RuntimeError(f"pt_render failed: {rc}")
        e2e_paths += W * H * k
    barrier()
    e2e_t = time.perf_counter() - e0
    e2e_val = e2e_paths / e2e_t
    if dist:
        tt = torch.tensor([e2e_t], device=f"cuda:{local_rank}", dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        e2e_val = e2e_paths * world / float(tt.item())
    h2d = C.sizeof(N.JobDesc) + spp_total * 8
    d2h = W * H * 3 * 4

    if rank != 0:
        return
    peak = None
    peak_src = "fallback"
    if PEAKS.exists():
        try:
            peak = float(json.loads(PEAKS.read_text())["hbm_gbs"])
            peak_src = "measured"
        except (KeyError, ValueError):
            peak = None
    if peak is None:
        peak = FALLBACK_HBM_GBS
    stages = stage_roofline(prof, tot, peak)
    # the dominant stage (CUDA events on the library stream): traversal =
    # closest-hit, paired and shadow-ray launches (+ the shadow resolve)
    dom = max(("traversal", "shade"), key=lambda kk: stages[kk]["ms"])
    dom_ms = stages[dom]["ms"]
    achieved = stages[dom]["achieved_gbs"]
    trav_launches = prof["trace"][1] + prof["shadow"][1]
    launches = sum(v[1] for v in prof.values())
    step_bytes_gbs = tot["bytes"] / (t_dev / 1e3) / 1e9
    ncu_bytes = NCU_TRAVERSAL_BYTES_PER_STEP.get((args.workload, wl["est"])) if k == 16 else None
    line = {
        "metric": "paths/s", "value": value, "unit": "paths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_dev / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator, no assets)",
        "config": {"workload": wl["desc"], "step": f"{k} spp x {W}x{H} px = {W * H * k} paths",
                   "estimator": wl["est_name"], "triangles": info["triangles"], "bvh4_nodes": info["bvh4_nodes"],
                   "bvh": "BVH4 collapsed from the reference's own trees (the library default)",
                   "l2": "inputs larger than L2: BVH + leaves "
                         f"{info['device_bytes'] / 1e6:.0f} MB and ~{tot['bytes'] / args.steps / 1e9:.1f} GB of "
                         "queue traffic per step (L2 129 MB)",
                   "parallelism": f"replicas x{world} (sample ranges per rank)"},
        "rays_per_s": (tot["rays"] + tot["shadow"]) * world / t_max,
        "e2e": {"value": e2e_val, "unit": "paths/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm",
                     "kernel": ("k_trace_closest / k_trace_pair / k_trace_shadow + k_shadow_resolve (traversal stage)"
                                if dom == "traversal" else "k_shade (shade stage)"),
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src,
                     "traffic": (ncu_bytes if ncu_bytes and dom == "traversal" else None),
                     "traffic_unit": "bytes per step: ncu dram__bytes_read.sum + dram__bytes_write.sum summed over "
                                     "the traversal stage's launches of one step (closest, paired, shadow, resolve; "
                                     "achieved is per step too: the stage's algorithmic bytes per step over its "
                                     "time per step)",
                     "algorithmic_bytes_per_step": stages[dom]["bytes"] / args.steps,
                     "algorithmic_bytes_note": "; ".join(f"{u} B per {c}" for c, u in STAGE_UNIT_BYTES[dom].items()),
                     "launches_per_step": trav_launches / args.steps if dom == "traversal" else None,
                     "stages": stages,
                     "counts_per_step": {kk: tot[kk2] / args.steps for kk, kk2 in
                                         (("paths", "paths"), ("segments", "segments"), ("rays", "rays"),
                                          ("shadow_rays", "shadow"), ("film_pixel_waves", "film_pixel_waves"))},
                     "note": f"stage share {dom_ms / sum(v[0] for v in prof.values()):.2f}; "
                             f"whole-step queue bytes (192 B per vertex + 88 B per shadow ray + 24 B per path) "
                             f"{step_bytes_gbs:.1f} GB/s; the traversal is bound by dependent node-load "
                             "latency, not bandwidth (L2 hit rate and warp efficiency in the committed ncu summary)"},
        "stage_ms": {kk: round(v[0], 3) for kk, v in prof.items()},
        "clocks": clk.summary(),
        "wall_s": wall,
    }
    if world == 1 and not args.no_rmse:
        line["rmse"] = converged_rmse(r, sid, cam, wl, k)
    if world == 1 and not args.no_forms:
        # the same job at twice the samples per call: two waves per call that
        # overlap on two queue sets (device time, not profiled)
        k2 = 2 * k
        n2 = max(1, args.steps // 2)
        chunks2 = max(1, spp_total // k2)

        def job2(step):
            c2 = sample_chunk(step, 0, 1, chunks2)
            return N.job_desc(sid, cam, W, H, wl["sx"], wl["sy"], wl["depth"], rr_start=wl["rr"],
                              estimator=wl["est"], sampler=wl["sampler"], env_sampling=wl["env"], seed=1,
                              spp_begin=c2 * k2, spp_end=c2 * k2 + k2)
        r.render_device(job2(0), film.data_ptr(), sync=True)
        t2, p2 = 0.0, 0
        for i in range(n2):
            st = r.render_device(job2(1 + i), film.data_ptr(), sync=False, stats=True)
            t2 += st.ms
            p2 += st.paths
        line["per_call"] = {"spp_per_call": k2, "paths_per_s": p2 / (t2 / 1e3), "unit": "paths/s", "calls": n2,
                            "note": "same job, two overlapped waves per call, device time"}
        # the same steps through the opt-in SAH trees (same hits, other tree)
        r.set_bvh_builder(N.BVH_BUILD_SAH)
        sid_sah = r.upload(sc)
        r.set_bvh_builder(N.BVH_BUILD_HOST)
        for i in range(args.warmup):
            r.render_device(job_for(i, sid_sah), film.data_ptr(), sync=True)
        t_sah, p_sah = 0.0, 0
        for i in range(args.steps):
            st = r.render_device(job_for(args.warmup + i, sid_sah), film.data_ptr(), sync=False, stats=True)
            t_sah += st.ms
            p_sah += st.paths
        r.release(sid_sah)
        line["bvh_variants"] = {"reference_tree": value, "sah_tree": p_sah / (t_sah / 1e3),
                                "unit": "paths/s",
                                "note": "PT_BVH_BUILD_SAH: binned-SAH BVH4, same steps and samples, device time"}
    if world == 1 and args.estimator == "ref_nee":
        # the same steps with NEE+MIS and the luminance alias table (device time)
        wm = workload(args.workload, "nee_mis")

        def job_mis(step):
            chunk = sample_chunk(step, 0, 1, max(1, spp_total // k))
            return N.job_desc(sid, cam, W, H, wm["sx"], wm["sy"], wm["depth"], rr_start=wm["rr"],
                              estimator=wm["est"], sampler=wm["sampler"], env_sampling=wm["env"], seed=1,
                              spp_begin=chunk * k, spp_end=chunk * k + k)
        for i in range(args.warmup):
            r.render_device(job_mis(i), film.data_ptr(), sync=True)
        t_m, p_m, r_m = 0.0, 0, 0
        for i in range(args.steps):
            st = r.render_device(job_mis(args.warmup + i), film.data_ptr(), sync=False, stats=True)
            t_m += st.ms
            p_m += st.paths
            r_m += st.rays + st.shadow_rays
        line["nee_mis"] = {"estimator": wm["est_name"], "paths_per_s": p_m / (t_m / 1e3),
                           "rays_per_s": r_m / (t_m / 1e3), "unit": "paths/s",
                           "note": "same scene, steps and sample streams, device time"}
    if world == 1 and not args.no_forms:
        fs, big, build_s, upload_s = form_scenes(r, with_big=True)
        forms = {"scene_build_s": build_s,
                 "big_scene_upload_s": dict(upload_s, triangles=5242880)}
        # the persistent form of the config-3 mix runs ~5x longer than the
        # graph form (about two minutes), so it is opt-in here
        forms["batched"] = run_batched(r, fs, args.batch_jobs, persistent=args.persistent_config3)
        # the regime batching exists for: many jobs far below one GPU's worth
        # of paths each (same scenes and cameras, smaller frames and spp)
        forms["batched_small_jobs"] = run_batched(r, fs, args.batch_jobs, seed=13, res=(64, 256), spp=(4, 32),
                                                  tune_sample=32, tune_spp=32)
        forms["served"] = run_served(r, fs, big, args.serve_seconds, args.serve_rate, pass_spp=args.serve_pass_spp,
                                     pass_paths=args.serve_pass_paths)
        if args.config4_seconds > 0:
            forms["served_config4"] = run_served_config4(r, fs, big, args.config4_seconds, 20.0,
                                                         args.config4_drain)
            forms["served_config4_saturating"] = run_served_config4(r, fs, big, 5.0, 200.0, args.config4_drain,
                                                                    seed=15)
        line["forms"] = forms
    if world == 1 and not args.no_forms:
        # configs 0 and 2 (Cornell, material divergence) at full size
        others = [n for n in ("cornell", "divergence") if n != args.workload]
        line["full_frames"] = run_full_frames(r, others, not args.no_cpu_baseline, os.cpu_count() or 1)
    if not args.no_cpu_baseline:
        from oracle import pyoracle as O

        threads = os.cpu_count() or 1
        osc = O.OracleScene(sc)
        v, sample, dt = cpu_paths_per_sec(osc, cam, wl, wl["est"], threads)
        line["cpu_baseline"] = {"value": v, "unit": "paths/s", "cores": threads, "kind": "port",
                                "estimator": wl["est_name"],
                                "sample": sample + f" ({dt:.1f} s); the reference integrator's CPU restatement "
                                                   "oracle/pt_oracle.cpp (recursive getRayColor for REF_NEE)"}
        if "nee_mis" in line:
            wm = workload(args.workload, "nee_mis")
            vm, sm, dtm = cpu_paths_per_sec(osc, cam, wm, wm["est"], threads)
            line["nee_mis"]["cpu_paths_per_s"] = vm
            line["nee_mis"]["cpu_sample"] = sm + f" ({dtm:.1f} s); the oracle's iterative NEE+MIS, {threads} threads"
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch

        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
