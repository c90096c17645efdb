#!/usr/bin/env python3
"""Benchmark of the GB300 spatial-statistics path: neighbour pairs/s.

Default workload ("tip20m", the plain method on an atom-probe tip): 20,000,000
ions in a truncated cone (apex radius 30 nm, half-angle 10 deg, length 200 nm;
density follows from N and the geometry, 13.42 nm^-3), Poisson matrix plus
2,000 Gaussian solute clusters (sigma 1.5 nm, 50 members, species 1/2 at
70/30 %), three iid minority species -- six species in all.  One step is the
two passes the reference needs for that workload (it has one bin width
per run): all 36 pairwise RDFs to R = 2.0 nm in 0.01 nm bins, then kNN
k = 1..10 for all 36 pairs in 0.005 nm bins, both with centres excluded within
R of the triangulated cone surface.  A neighbour pair is one in-ball
(centre, neighbour) pair of one pass.

`value` times the passes on a resident cloud (CUDA events on the launching
stream); `e2e` times the public C ABI from pinned host buffers (upload, hull,
both passes, result fetch).  The cloud (320 MB of cell-sorted records) is
larger than L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
Under torchrun each rank runs an independent replica (the path does not
shard); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "neighbour pairs/s"
UNIT = "pairs/s"
BYTES_PER_PAIR = 16  # one float4 {x, y, z, type} neighbour record per in-ball pair


# ------------------------------------------------------------------ workloads
def workload(name):
    from paraprobe_gb300 import synth
    if name in ("tip20m", "tip10m"):
        n = 20_000_000 if name == "tip20m" else 10_000_000
        rho = 20_000_000 / synth.cone_volume(30.0, 10.0, 200.0)
        length = 200.0 if name == "tip20m" else synth.cone_length_for(n, rho, 30.0, 10.0)
        spec = synth.cone_specimen(n=n, r_apex=30.0, half_angle_deg=10.0, length=length,
                                   n_clusters=2000 * n // 20_000_000, sigma=1.5, members=50,
                                   cluster_p=(0.7, 0.3), iid=(0.02, 0.01, 0.005), nspecies=6,
                                   seed=20261205)
        types = list(range(1, 7))
        trg = [[a] for a in types for b in types]
        env = [[b] for a in types for b in types]
        runs = [dict(flags=1, hist=(0.0, 0.01, 2.0), k=[]),
                dict(flags=8, hist=(0.0, 0.005, 2.0), k=list(range(10, 0, -1)))]
        cfg = {"workload": f"{name}: {n // 1_000_000}M-ion clustered truncated cone (r_apex 30 nm, 10 deg, "
                           f"L {length:.1f} nm), 6 species, 36 pair tasks; pass 1 RDF R=2.0/0.01, pass 2 kNN "
                           "k=1..10 R=2.0/0.005, hull-distance exclusion",
               "ions": n, "tasks": 36, "R_nm": 2.0}
    elif name == "tip150m":
        # the 150M-ion tip: apex r 50 nm, 12 deg, L 400 nm, 8 species,
        # 5000 clusters; RDF and kNN k = 1..20 for all 64 pairs in one pass
        # (one bin geometry, 2.5 nm / 0.01 nm)
        n = 150_000_000
        spec = synth.cone_specimen(n=n, r_apex=50.0, half_angle_deg=12.0, length=400.0, n_clusters=5000,
                                   sigma=1.5, members=50, cluster_p=(0.7, 0.3),
                                   iid=(0.02, 0.01, 0.005, 0.005, 0.002), nspecies=8, seed=20261208)
        types = list(range(1, 9))
        trg = [[a] for a in types for b in types]
        env = [[b] for a in types for b in types]
        runs = [dict(flags=1 | 8, hist=(0.0, 0.01, 2.5), k=list(range(20, 0, -1)))]
        cfg = {"workload": "tip150m: 150M-ion clustered truncated cone (r_apex 50 nm, 12 deg, L 400 nm), 8 species, "
                           "5000 clusters, 64 pair tasks; one pass RDF + kNN k=1..20, R=2.5/0.01, hull-distance "
                           "exclusion",
               "ions": n, "tasks": 64, "R_nm": 2.5}
    elif name == "tip8sp10m":
        # a 10M-ion cut of the 150M-ion tip's kind (same apex, angle, density,
        # cluster density, species and analyses), for profiling its kernels
        n = 10_000_000
        rho = 150_000_000 / synth.cone_volume(50.0, 12.0, 400.0)
        length = synth.cone_length_for(n, rho, 50.0, 12.0)
        spec = synth.cone_specimen(n=n, r_apex=50.0, half_angle_deg=12.0, length=length, n_clusters=333,
                                   sigma=1.5, members=50, cluster_p=(0.7, 0.3),
                                   iid=(0.02, 0.01, 0.005, 0.005, 0.002), nspecies=8, seed=20261208)
        types = list(range(1, 9))
        trg = [[a] for a in types for b in types]
        env = [[b] for a in types for b in types]
        runs = [dict(flags=1 | 8, hist=(0.0, 0.01, 2.5), k=list(range(20, 0, -1)))]
        cfg = {"workload": f"tip8sp10m: 10M-ion cut (L {length:.1f} nm) of the 150M-ion tip's kind (r_apex 50 nm, "
                           "12 deg), 8 species, 64 pair tasks; one pass RDF + kNN k=1..20, R=2.5/0.01",
               "ions": n, "tasks": 64, "R_nm": 2.5}
    elif name == "cyl1m":
        spec = synth.cylinder_specimen(n=1_000_000, radius=10.0, height=63.66, fractions=(0.90, 0.08, 0.02),
                                       seed=20261204)
        trg, env = [[2]], [[1, 2, 3]]
        runs = [dict(flags=1 | 8, hist=(0.0, 0.01, 1.0), k=[10, 5, 1])]
        cfg = {"workload": "cyl1m: 1M uniform ions in a cylinder (r 10 nm, h 63.66 nm), species 1 centres, "
                           "RDF R=1.0/0.01 + kNN k=1,5,10 against all species",
               "ions": 1_000_000, "tasks": 1, "R_nm": 1.0}
    else:
        raise SystemExit(f"unknown workload {name}")
    return spec, trg, env, runs, cfg


def tip_cloud(n, seed):
    """A clustered cone like the tip20m one: same apex, angle, density
    (13.42 nm^-3) and cluster density, length shortened to hold n ions."""
    from paraprobe_gb300 import synth
    rho = 20_000_000 / synth.cone_volume(30.0, 10.0, 200.0)
    length = synth.cone_length_for(n, rho, 30.0, 10.0)
    return synth.cone_specimen(n=n, r_apex=30.0, half_angle_deg=10.0, length=length,
                               n_clusters=max(1, round(2000 * n / 20_000_000)), sigma=1.5, members=50,
                               cluster_p=(0.7, 0.3), iid=(0.02, 0.01, 0.005), nspecies=6, seed=seed), length


# --------------------------------------------------------------------- helpers
def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_bytes(workload_name, kernel):
    """DRAM bytes (read + write) per launch of `kernel` on the workload, from
    the committed ncu summary profiles/dram_traffic.md, if it lists them."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        parts = [x.strip().strip("`") for x in line.strip().strip("|").split("|")]
        if len(parts) >= 3 and parts[0] == workload_name and parts[1] == kernel:
            try:
                return float(parts[2])
            except ValueError:
                continue
    return None


class Clocks:
    """nvidia-smi sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = list(csv.reader(io.StringIO(open(self.path).read())))
        os.unlink(self.path)
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def reduce_max(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------ CPU (oracle)
# One sample rule for every CPU figure (the GPU arm's cpu_baseline leg and the
# reference arm): the ions whose key (uniform on [0, 1), numpy seed 7) is
# below the workload's fraction may be centres; the whole cloud stays the
# environment.  The same mask drives the GPU parity check of the GPU arm.
CPU_SAMPLE = {"tip20m": 0.02, "tip10m": 0.04, "cyl1m": 1.0, "tip150m": 0.002, "tip8sp10m": 0.02}


def sample_mask(n, frac):
    if frac >= 1.0:
        return None
    return (np.random.default_rng(7).random(n) < frac).astype(np.uint8)


def cpu_leg(name, steps, warmup, threads):
    """The oracle port (the reference's algorithm: z-slabs, per-slab KD-trees,
    per-centre statistics; OpenMP on `threads` host threads) on the workload's
    centre sample.  Times the three phases the reference reports separately:
    Ion2SurfThreadparallelDistancing (hull distance of every ion, once),
    ThreadparallelKDTreeConstruct (decomposition and KD-trees, once per pass)
    and DescrStatsThreadparallelCompute (the statistics over the sampled
    centres).  Returns (record, bins of each pass)."""
    from oracle import oracle as O
    spec, trg, env, runs, cfg = workload(name)
    n = spec.xyz.shape[0]
    frac = CPU_SAMPLE[name]
    mask = sample_mask(n, frac)
    rp = max(2.0, max(r["hist"][2] for r in runs))
    t0 = time.perf_counter()
    surf = O.surface_distance(spec.xyz, spec.hull, rp, nthreads=threads)
    surf_s = time.perf_counter() - t0

    def step():
        return [O.spatstat(spec.xyz, spec.labels, surf, *r["hist"], r["flags"], trg, env, r["k"],
                           centre_mask=mask, nthreads=threads) for r in runs]

    for _ in range(warmup):
        step()
    pairs, comp_s, build_s, outs = 0, 0.0, 0.0, []
    for _ in range(steps):
        outs = step()
        pairs += sum(o["pairs"] for o in outs)
        comp_s += sum(o["compute_s"] for o in outs)
        build_s += sum(o["build_s"] for o in outs)
    per_step_pairs = pairs // max(steps, 1)
    stat_s = comp_s / max(steps, 1)
    build_step_s = build_s / max(steps, 1)
    # one whole step of the reference (every centre, every pass: each pass is
    # a separate reference run with its own hull distancing and KD-trees)
    full_stat_s = stat_s / frac
    full_s = len(runs) * surf_s + build_step_s + full_stat_s
    rec = {"value": pairs / max(comp_s, 1e-9), "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"oracle port (z-slab KD-trees + OpenMP, restating the reference) over "
                     f"{frac * 100:g}% of the ions as candidate centres (numpy seed 7 keys), whole cloud as "
                     f"environment; {steps} timed step(s) after {warmup} warm-up; value = statistics phase",
           "sample_fraction": frac, "pairs_per_step": int(per_step_pairs),
           "phases": {"surface_distancing_s": round(surf_s, 4),
                      "surface_distancing_ions_per_s": n / max(surf_s, 1e-9),
                      "kdtree_build_s_per_step": round(build_step_s, 4),
                      "kdtree_build_ions_per_s": n * len(runs) / max(build_step_s, 1e-9),
                      "statistics_s_per_step": round(stat_s, 4),
                      "statistics_pairs_per_s": per_step_pairs / max(stat_s, 1e-9)},
           "full_step_estimate": {"seconds": round(full_s, 3),
                                  "pairs": int(per_step_pairs / frac),
                                  "pairs_per_s": per_step_pairs / frac / full_s,
                                  "rule": "passes x hull distancing + KD-tree builds + statistics / sample "
                                          "fraction"}}
    return rec, [o["bins"] for o in outs]


def cpu_leg_subprocess(name, steps, warmup):
    """cpu_leg in a fresh interpreter (no CUDA context, no torch), so that the
    GPU arm's CPU figure is taken exactly as the reference arm's."""
    fd, path = tempfile.mkstemp(suffix=".npz")
    os.close(fd)
    try:
        subprocess.run([sys.executable, os.path.abspath(__file__), "--cpu-leg", "--workload", name,
                        "--steps", str(steps), "--warmup", str(warmup), "--cpu-out", path],
                       check=True, stdout=subprocess.DEVNULL)
        z = np.load(path, allow_pickle=False)
        rec = json.loads(str(z["record"]))
        bins = [z[f"bins{i}"] for i in range(int(z["npass"]))]
        return rec, bins
    finally:
        os.unlink(path)


def cpu_leg_main(args):
    threads = os.cpu_count() or 1
    rec, bins = cpu_leg(args.workload, args.steps, args.warmup, threads)
    np.savez(args.cpu_out, record=json.dumps(rec), npass=len(bins), **{f"bins{i}": b for i, b in enumerate(bins)})


# ------------------------------------------------------------------ GPU arm
def run_gpu(args):
    import torch
    from paraprobe_gb300 import build as B
    B.build()
    from paraprobe_gb300 import native as N

    world, rank, local, pg = dist_setup()
    torch.cuda.set_device(local)
    spec, trg, env, runs, cfg = workload(args.workload)
    n = spec.xyz.shape[0]
    ctx = N.Context(local)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    # untimed: the project autotuner picks cell edge and block tile on a
    # sample of centres of the heaviest pass
    heavy = runs[-1]
    ctx.tasks(trg, env)
    ctx.hist(*heavy["hist"])
    if args.tuning:
        # fixed tuning (ratio:tile code), e.g. for a profiler run with a
        # predictable launch sequence
        ratio, tile = float(args.tuning.split(":")[0]), int(args.tuning.split(":")[1], 0)
        ctx.tuning(cid, ratio, tile)
    else:
        ratio, tile = ctx.autotune(cid, heavy["flags"], heavy["k"], sample=200000)

    pass_kernel = ["" for _ in runs]
    pass_tests = [0 for _ in runs]

    def step():
        pairs = 0
        kms = []
        for i, r in enumerate(runs):
            ctx.tasks(trg, env)
            ctx.hist(*r["hist"])
            ctx.run(cid, r["flags"], r["k"], stream=sh)
            ctx.fetch()
            pairs += ctx.stats()["pairs"]
            kms.append(ctx.last_kernel_ms())
            pass_kernel[i] = ctx.last_kernel()
        return pairs, kms

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clk = Clocks(local)
    clk.start()
    barrier(pg)
    launches0 = N.kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    tot_pairs = 0
    per_pass_ms = [[] for _ in runs]
    per_pass_pairs = [0 for _ in runs]
    for _ in range(args.steps):
        p, kms = step()
        tot_pairs += p
        for i, m in enumerate(kms):
            per_pass_ms[i].append(m)
    e1.record(stream)
    torch.cuda.synchronize()
    launches = N.kernel_launches() - launches0
    elapsed = e0.elapsed_time(e1) / 1e3
    barrier(pg)
    clocks = clk.stop()
    # pairs per pass (same every step); FP64 audit of each pass's bins on
    # 20000 evenly spaced centres (untimed)
    audits = []
    for i, r in enumerate(runs):
        ctx.tasks(trg, env)
        ctx.hist(*r["hist"])
        ctx.run(cid, r["flags"], r["k"], stream=sh)
        ctx.fetch()
        per_pass_pairs[i] = ctx.stats()["pairs"]
        pass_tests[i] = ctx.run_tests()
        au = ctx.fp64_audit(cid, max_centres=20000, cap=1 << 16)
        audits.append({"bins": f"{r['hist'][1]} nm", "pairs": au["pairs"],
                       "max_abs_err_nm": au["max_abs_err"], "max_rel_err": au["max_rel_err"],
                       "bin_disagreements": au["bin_disagreements"],
                       "in_ball_disagreements": au["set_disagreements"]})
    t_max = reduce_max(pg, elapsed)
    value = tot_pairs * world / t_max

    # ---- end to end through the C ABI from pinned host memory
    xyz_pin = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    xyz_pin.numpy()[:] = spec.xyz
    lab_pin = torch.empty((n,), dtype=torch.uint8, pin_memory=True)
    lab_pin.numpy()[:] = spec.labels
    tri = np.ascontiguousarray(spec.hull, dtype=np.float32)

    def e2e_step():
        c = ctx.upload(xyz_pin.numpy(), lab_pin.numpy())
        ctx.tuning(c, ratio, tile)
        ctx.hull(c, tri, 2.0)
        pairs = 0
        d2h = 0
        for r in runs:
            ctx.tasks(trg, env)
            ctx.hist(*r["hist"])
            ctx.run(c, r["flags"], r["k"], stream=sh)
            out = ctx.fetch()
            d2h += out.nbytes
            pairs += ctx.stats()["pairs"]
        ctx.free(c)
        return pairs, d2h

    e2e_step()
    torch.cuda.synchronize()
    barrier(pg)
    t0 = time.perf_counter()
    e_pairs = 0
    d2h = 0
    e_steps = max(3, min(args.steps, 10))
    for _ in range(e_steps):
        p, d2h = e2e_step()
        e_pairs += p
    torch.cuda.synchronize()
    e_el = reduce_max(pg, time.perf_counter() - t0)
    e2e = {"value": e_pairs * world / e_el, "unit": UNIT,
           "h2d_bytes_per_step": int(n * 12 + n + tri.nbytes + 2 * len(trg) * 8 * 4 * len(runs)),
           "d2h_bytes_per_step": int(d2h), "steps": e_steps,
           "includes": "upload + device grid build + hull distance + all passes + result fetch"}

    # ---- roofline of the dominant kernel (the pass with the longest launch),
    # measured live with CUDA events around each launch on its stream
    peak, kind = peaks()
    per_pass = []
    for i in range(len(runs)):
        ms = statistics.mean(per_pass_ms[i])
        ach = BYTES_PER_PAIR * per_pass_pairs[i] / (ms / 1e3) / 1e9
        per_pass.append({"kernel": pass_kernel[i], "ms": round(ms, 3), "pairs": int(per_pass_pairs[i]),
                         "tests_per_pair": round(pass_tests[i] / max(per_pass_pairs[i], 1), 3),
                         "achieved": round(ach, 1), "frac": round(ach / peak, 4),
                         "traffic": traffic_bytes(args.workload, pass_kernel[i])})
    dom = max(range(len(runs)), key=lambda i: per_pass[i]["ms"])
    all_s = sum(p["ms"] for p in per_pass) / 1e3
    all_ach = BYTES_PER_PAIR * sum(per_pass_pairs) / all_s / 1e9
    roof = {"bound": "hbm", "achieved": per_pass[dom]["achieved"], "peak": peak, "unit": "GB/s",
            "frac": per_pass[dom]["frac"], "peak_kind": kind, "traffic": per_pass[dom]["traffic"],
            "kernel": per_pass[dom]["kernel"], "per_pass": per_pass,
            "all_passes": {"achieved": round(all_ach, 1), "frac": round(all_ach / peak, 4)},
            "algorithmic_bytes_per_pair": BYTES_PER_PAIR}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(cfg, passes=len(runs), pairs_per_step=int(tot_pairs // args.steps),
                           tuning={"cell_edge_nm": round(cfg["R_nm"] / ratio, 4), "tile": tile},
                           l2="inputs larger than L2 (cell-sorted cloud 16 B/ion), no flush",
                           parallelism=f"replicas x{world}"),
            "roofline": roof, "e2e": e2e, "gpu_launches": int(launches), "clocks": clocks,
            "fp64_audit": audits}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # the oracle on the workload's centre sample (a fresh process), then
        # the GPU pass on the same sample: the bins must be identical
        line.update(guarded("cpu_baseline", lambda: parity_leg(ctx, cid, sh, spec, trg, env, runs, args)))
    if not args.no_batched and args.workload == "tip150m":
        line.update(guarded("batched", lambda: batched_leg_large(ctx, cid, spec, trg, env, runs[0], torch, stream,
                                                                 per_pass_pairs[0], per_pass_ms[0])))
    ctx.free(cid)
    if not args.no_batched and args.workload != "tip150m":
        line.update(guarded("batched", lambda: batched_leg(ctx, torch, stream)))
    if not args.no_served:
        line.update(guarded("served", lambda: served_leg(ctx)))
    if not args.no_large and args.workload != "tip150m" and world == 1:
        del spec
        line.update(guarded("large", lambda: large_leg(ctx, torch, stream, args)))
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


def guarded(key, fn):
    """An optional leg of the bench: {key: its result} (or the keys it returns
    itself, when it returns several), or {key: {"error": ...}} when it fails,
    so that a failing leg never costs the bench line."""
    try:
        out = fn()
        return out if key in out and isinstance(out[key], dict) and len(out) > 1 else {key: out}
    except Exception as e:  # noqa: BLE001 -- reported in the line
        return {key: {"error": f"{type(e).__name__}: {e}"[:300]}}


def parity_leg(ctx, cid, sh, spec, trg, env, runs, args):
    """The oracle on the workload's centre sample (cpu_baseline) and the GPU
    passes on the same sample (parity): {"cpu_baseline": ..., "parity": ...}."""
    n = spec.xyz.shape[0]
    rec, cpu_bins = cpu_leg_subprocess(args.workload, steps=2, warmup=1)
    mask = sample_mask(n, CPU_SAMPLE[args.workload])
    checks = []
    for i, r in enumerate(runs):
        ctx.tasks(trg, env)
        ctx.hist(*r["hist"])
        ctx.run(cid, r["flags"], r["k"], stream=sh, centre_mask=mask)
        g = ctx.fetch()
        st = ctx.stats()
        same = g.shape == cpu_bins[i].shape and bool(np.array_equal(g, cpu_bins[i]))
        checks.append({"pass": i + 1, "kernel": ctx.last_kernel(), "centres": st["centres"],
                       "pairs": st["pairs"], "bins": int(g.size), "bins_identical": same,
                       "bins_differing": int(np.count_nonzero(g != cpu_bins[i])) if g.shape == cpu_bins[i].shape
                       else int(g.size)})
    parity = {"against": "oracle port on the cpu_baseline sample (same centre mask, same cloud)",
              "sample_fraction": CPU_SAMPLE[args.workload],
              "centres": sum(c["centres"] for c in checks), "pairs": sum(c["pairs"] for c in checks),
              "bins_identical": all(c["bins_identical"] for c in checks), "passes": checks}
    return {"cpu_baseline": rec, "parity": parity}


# ---------------------------------------------------- batched (null model + ROIs)
def batched_leg(ctx, torch, stream):
    """Batched realisations: a 5M-ion clustered tip, 256 label shuffles (own seeds)
    and 64 spherical ROIs (radius log-uniform 5-40 nm, centres uniform in the
    tip) plus the measured labels, RDF to R = 1.5 nm and kNN k = 1..8 in
    0.01 nm bins for all 36 pair tasks -- every realisation in one persistent
    launch.  Compared with the plain single-query path on the same cloud."""
    from concurrent.futures import ThreadPoolExecutor
    from paraprobe_gb300 import native as N
    spec, length = tip_cloud(5_000_000, seed=20261206)
    n = spec.xyz.shape[0]
    types = list(range(1, 7))
    trg = [[a] for a in types for b in types]
    env = [[b] for a in types for b in types]
    hist = (0.0, 0.01, 1.5)
    ks = list(range(8, 0, -1))
    flags = N.PP_RDF | N.PP_MKNN
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        sets = list(ex.map(lambda r: N.shuffle_labels(spec.labels, 1000 + r), range(256)))
    sets_dev = torch.from_numpy(np.stack(sets)).to("cuda")  # resident in HBM
    rng = np.random.default_rng(20261207)
    rois = []
    tn = np.tan(np.radians(10.0))
    while len(rois) < 64:
        z = rng.uniform(0, length)
        rz = 30.0 + z * tn
        x, y = rng.uniform(-rz, rz, 2)
        if x * x + y * y <= rz * rz:
            rois.append([x, y, z, float(np.exp(rng.uniform(np.log(5.0), np.log(40.0))))])
    rois = np.asarray(rois, dtype=np.float32)
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(*hist)
    ratio, tile = ctx.autotune(cid, flags, ks, sample=100000)
    # plain single-query path, same cloud and passes (one realisation)
    for _ in range(2):
        ctx.run(cid, flags, ks, stream=stream.cuda_stream)
        ctx.fetch()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 3
    plain_pairs = 0
    for _ in range(reps):
        ctx.run(cid, flags, ks, stream=stream.cuda_stream)
        ctx.fetch()
        plain_pairs += ctx.stats()["pairs"]
    plain = plain_pairs / (time.perf_counter() - t0)

    def batched_call():
        ctx.tasks(trg, env)  # drops the cached pair lists: geometry is rebuilt inside the timed call
        ctx.run_batched(cid, flags, ks, include_original=True, label_sets=sets_dev.data_ptr(), nsets=len(sets),
                        rois=rois, stream=stream.cuda_stream)
        nreal = ctx.batched_count()
        pairs = sum(ctx.batched_stats(r)["pairs"] for r in range(nreal))
        return nreal, pairs

    batched_call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nreal, pairs = batched_call()
    cold = time.perf_counter() - t0
    apply_ms = ctx.last_kernel_ms()
    graph = ctx.batched_graph()
    ctx.free(cid)
    return {"workload": "5M-ion clustered tip (as tip20m), 36 pair tasks, RDF + kNN k=1..8, "
                        "R=1.5 nm, 0.01 nm bins; 1 measured + 256 shuffled label sets + 64 ROIs",
            "realisations": nreal, "pairs": int(pairs), "value": pairs / cold, "unit": UNIT,
            "seconds": round(cold, 4), "apply_graph_ms": round(apply_ms, 3),
            "apply_value": pairs / (apply_ms * 1e-3) if apply_ms > 0 else None,
            "plain_single_query": plain, "ratio_vs_plain": (pairs / cold) / plain,
            "cuda_graph": graph,
            "tuning": {"cell_edge_nm": round(1.5 / ratio, 4), "tile": tile},
            "includes": "pair-list geometry, label gathers and layouts, masks, the realisation passes (one CUDA "
                        "graph: persistent RDF/count launch + 32-realisation kNN walk/bin launches), result fetch"}


def batched_leg_large(ctx, cid, spec, trg, env, run, torch, stream, plain_pairs, plain_ms):
    """The 150M-ion tip batched: the measured labels plus 32 label
    shuffles in one batched call on the resident 150M-ion cloud.  Its pair
    lists (about 10^11 pairs) exceed HBM, so they are built and applied a chunk
    of centres at a time.  Compared with the plain pass on the same cloud."""
    from paraprobe_gb300 import native as N
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        sets = list(ex.map(lambda r: N.shuffle_labels(spec.labels, 5000 + r), range(32)))
    sets_dev = torch.from_numpy(np.stack(sets)).to("cuda")
    del sets
    ctx.tasks(trg, env)
    ctx.hist(*run["hist"])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ctx.run_batched(cid, run["flags"], run["k"], include_original=True, label_sets=sets_dev.data_ptr(), nsets=32,
                    stream=stream.cuda_stream)
    nreal = ctx.batched_count()
    pairs = sum(ctx.batched_stats(r)["pairs"] for r in range(nreal))
    el = time.perf_counter() - t0
    apply_ms = ctx.last_kernel_ms()
    plain = plain_pairs / (statistics.mean(plain_ms) * 1e-3)
    return {"workload": "tip150m batched: 1 measured + 32 shuffled label sets, RDF + kNN k=1..20, "
                        "R=2.5/0.01, 64 pair tasks, pair lists built and applied in centre chunks",
            "realisations": nreal, "pairs": int(pairs), "value": pairs / el, "unit": UNIT, "seconds": round(el, 3),
            "apply_graph_ms": round(apply_ms, 3), "cuda_graph": ctx.batched_graph(),
            "plain_single_query": plain, "ratio_vs_plain": (pairs / el) / plain,
            "includes": "pair-list geometry (count pass, per-chunk emit), label gathers and layouts, all "
                        "realisation passes, result fetch"}


# ------------------------------------------------------------- the largest tip
def large_leg(ctx, torch, stream, args):
    """The largest single-GPU workload (tip150m: 150M ions, 8 species, 64
    tasks, RDF + kNN k = 1..20 at R = 2.5 / 0.01 nm in one pass) on its own:
    autotuned plain pass, timed on the resident cloud; its bins against the
    oracle on the tip150m centre sample; then the measured labels with 32
    label shuffles batched alongside."""
    from paraprobe_gb300 import native as N
    spec, trg, env, runs, cfg = workload("tip150m")
    r = runs[0]
    n = spec.xyz.shape[0]
    sh = stream.cuda_stream
    cid = ctx.upload(spec.xyz, spec.labels)
    ctx.hull(cid, spec.hull, 2.0)
    ctx.tasks(trg, env)
    ctx.hist(*r["hist"])
    ratio, tile = ctx.autotune(cid, r["flags"], r["k"], sample=200000)
    for _ in range(2):
        ctx.run(cid, r["flags"], r["k"], stream=sh)
        ctx.fetch()
    steps = 3
    ms, kms = [], []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.run(cid, r["flags"], r["k"], stream=sh)
        e1.record(stream)
        ctx.fetch()
        ms.append(e0.elapsed_time(e1))
        kms.append(ctx.last_kernel_ms())
    pairs = ctx.stats()["pairs"]
    kernel = ctx.last_kernel()
    peak, kind = peaks()
    t = statistics.mean(ms) / 1e3
    out = {"workload": cfg["workload"], "ions": n, "value": pairs / t, "unit": UNIT, "ms_per_pass": round(t * 1e3, 2),
           "pairs": int(pairs), "kernel": kernel, "kernel_ms": round(statistics.mean(kms), 2),
           "roofline": {"achieved": round(BYTES_PER_PAIR * pairs / t / 1e9, 1), "peak": peak, "peak_kind": kind,
                        "frac": round(BYTES_PER_PAIR * pairs / t / 1e9 / peak, 4)},
           "tuning": {"cell_edge_nm": round(cfg["R_nm"] / ratio, 4), "tile": tile}}
    if not args.no_cpu_baseline:
        def parity():
            cpu_rec, cpu_bins = cpu_leg_subprocess("tip150m", steps=1, warmup=0)
            ctx.run(cid, r["flags"], r["k"], stream=sh, centre_mask=sample_mask(n, CPU_SAMPLE["tip150m"]))
            g = ctx.fetch()
            st = ctx.stats()
            return {"parity": {"against": "oracle port on the tip150m CPU sample (same centre mask, same cloud)",
                               "sample_fraction": CPU_SAMPLE["tip150m"], "centres": st["centres"],
                               "pairs": st["pairs"], "bins": int(g.size), "kernel": ctx.last_kernel(),
                               "bins_identical": bool(g.shape == cpu_bins[0].shape and
                                                      np.array_equal(g, cpu_bins[0]))},
                    "cpu_baseline": cpu_rec}
        out.update(guarded("parity", parity))
    if not args.no_batched:
        out.update(guarded("batched", lambda: batched_leg_large(ctx, cid, spec, trg, env, r, torch, stream, pairs, ms)))
    ctx.free(cid)
    return out


# ------------------------------------------------------------- served queries
def served_leg(ctx, nq=240, rate=200.0):
    """Serving: six resident clouds (0.1M .. 50M ions, tips like
    tip20m); queries arrive as a Poisson stream at `rate`/s, each with
    a random cloud, R ~ U[0.5, 3.0] nm, k ~ U[1, 20] and a random species pair
    (RDF + kNN, 0.01 nm bins).  Continuous batching on 4 worker streams,
    admission by HBM footprint; queries waiting on the same cloud run as one
    merged pass; compared with the same queries run one at a time through
    pp_run."""
    from paraprobe_gb300 import native as N
    sizes = (100_000, 1_000_000, 5_000_000, 10_000_000, 20_000_000, 50_000_000)
    clouds = []
    for i, n in enumerate(sizes):
        spec, _ = tip_cloud(n, seed=20261300 + i)
        c = ctx.upload(spec.xyz, spec.labels)
        ctx.hull(c, spec.hull, 2.0)
        ctx.prepare(c, 0.5, 3.0)
        clouds.append(c)
        del spec
    rng = np.random.default_rng(20261208)
    qs = []
    for _ in range(nq):
        c = clouds[rng.integers(0, len(clouds))]
        R = float(np.float32(rng.uniform(0.5, 3.0)))
        k = int(rng.integers(1, 21))
        a, b = (int(x) for x in rng.integers(1, 7, size=2))
        qs.append((c, N.PP_RDF | N.PP_MKNN, (0.0, 0.01, R), [[a]], [[b]], [k]))
    free = 0
    try:
        import torch
        free = torch.cuda.mem_get_info()[0]
    except Exception:
        pass
    budget = int(max(2 << 30, free * 0.6))

    def stream(arrival, seed):
        """The queries as a Poisson stream at `arrival`/s through a fresh server."""
        gaps = np.random.default_rng(seed).exponential(1.0 / arrival, size=nq)
        srv = N.Server(ctx, slots=4, budget_bytes=budget)
        for q in qs[:4]:  # warm the workers
            srv.wait(srv.submit(*q))
        t0 = time.perf_counter()
        tickets, t_next = [], t0
        for q, g in zip(qs, gaps):
            t_next += g
            dt = t_next - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            try:
                tickets.append(srv.submit(*q))
            except N.PPError:
                pass
        got = 0
        for t in tickets:
            got += srv.wait(t)[1]
        el = time.perf_counter() - t0
        st = srv.stats()
        npass, taken = srv.passes()
        srv.close()
        return tickets, got, el, st, npass, taken

    tickets, pairs, served_s, st, passes, taken = stream(rate, 20261209)
    # the same stream at a rate the server sustains (70% of the queries per
    # second it completed above): latency without a growing queue
    rate_ok = round(0.7 * len(tickets) / served_s, 1)
    t2, pairs2, s2, st2, passes2, taken2 = stream(rate_ok, 20261210)
    # the same queries one at a time through the plain path
    t0 = time.perf_counter()
    plain_pairs = 0
    for (c, f, h, tr, en, k) in qs:
        ctx.tasks(tr, en)
        ctx.hist(*h)
        ctx.run(c, f, k)
        ctx.fetch()
        plain_pairs += ctx.stats()["pairs"]
    plain_s = time.perf_counter() - t0
    for c in clouds:
        ctx.free(c)
    return {"workload": "6 resident tips (0.1M, 1M, 5M, 10M, 20M, 50M ions), Poisson 200/s, R~U[0.5,3] nm, "
                        "k~U[1,20], random species pair, RDF + kNN",
            "queries": len(tickets), "value": pairs / served_s, "unit": UNIT,
            "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "admitted": int(st["admitted"]) - 4,
            "rejected": int(st["rejected"]), "slots": 4, "budget_bytes": budget,
            "arrival_rate_per_s": rate, "served_queries_per_s": len(tickets) / served_s,
            "merged_passes": int(passes) - 4, "queries_per_pass": (taken - 4) / max(passes - 4, 1),
            "plain_single_query": plain_pairs / plain_s, "ratio_vs_plain": (pairs / served_s) / (plain_pairs / plain_s),
            "sustained": {"arrival_rate_per_s": rate_ok, "value": pairs2 / s2, "p50_ms": st2["p50_ms"],
                          "p99_ms": st2["p99_ms"], "served_queries_per_s": len(t2) / s2,
                          "merged_passes": int(passes2) - 4, "rejected": int(st2["rejected"])}}


# ------------------------------------------------------------ reference arm
def run_reference(args):
    """The reference's CPU algorithm (the oracle port; the reference's own
    units do not build on the Arm host) on all host cores, each step the
    workload's centre sample, with the same sample rule as the GPU arm's
    cpu_baseline leg."""
    world, rank, local, pg = dist_setup()
    if rank != 0:
        if pg is not None:
            pg.barrier()
            pg.destroy_process_group()
        return
    _, _, _, runs, cfg = workload(args.workload)
    threads = os.cpu_count() or 1
    rec, _ = cpu_leg(args.workload, args.steps, args.warmup, threads)
    value = rec["value"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": rec["phases"]["statistics_s_per_step"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference", "config": dict(cfg, passes=len(runs)), "cpu_baseline": rec,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    if pg is not None:
        pg.barrier()
        pg.destroy_process_group()


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="tip20m", choices=["tip20m", "tip10m", "cyl1m", "tip150m", "tip8sp10m"])
    ap.add_argument("--tuning", default=None, help="RATIO:TILE -- skip the autotuner, use this cell ratio and tile code")
    ap.add_argument("--cpu-leg", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--cpu-out", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched realisation leg")
    ap.add_argument("--no-served", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-large", action="store_true", help="skip the 150M-ion tip leg")
    args = ap.parse_args()
    if args.cpu_leg:
        cpu_leg_main(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
