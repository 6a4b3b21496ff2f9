#!/usr/bin/env python
"""Benchmark of the GB300 finite-volume RK stage.

Workload: the relativistic wind on 4096 x 1024 zones (64 radial blocks of
64 x 1024, r in [1, 10.0008]), gamma 4/3, PLM theta 1.5, HLLE, RK2, CFL 0.4,
seeded synthetic initial data. A step is one full RK2 step over every zone.

Reported (one JSON line from rank 0):
  value        zone-updates/s of the mixed-precision + learned-c2p-guess +
               graph-batched path (device-timed with CUDA events around the
               captured graphs; inputs resident in HBM)
  fp64         the plain FP64 path on the same workload, and the FP64 pipe
               fraction it reaches (against the FP64 FMA rate measured here)
  l1_density   L1 error of the comoving density of the mixed path against the
               FP64 path after the workload's 200 steps (the FP64 path equals
               the CPU oracle to 1e-12, so this is the error against the FP64
               oracle); l1_density_twice_the_steps: after 400;
               l1_density_after_run: after this run's steps
  errors_vs_fp64  relative L1 and Linf per conserved field, same comparison
  roofline     the dominant kernel of the headline path: algorithmic bytes per
               launch / its average CUDA-event duration, against measured HBM
  e2e          the same metric through the C ABI with host buffers: every step
               is one knc_advance_host call, which takes the whole state from
               pinned host memory and writes the new state back (uploads and
               downloads by chunks of blocks, beside the stages)
  batched_uneven  96 uneven blocks (nr 32..512, nq 64..256), RK3, both
               excision surfaces at 0.5c: mixed + learned + graph vs FP64
  learned_jet  the W = 100 jet on 2048 x 512 for its configured 200 steps:
               plain Newton from the reference's guess vs the learned guess,
               in the mixed path and in the FP64 path (iterations per zone,
               throughput, density L1 against the FP64 path)
  next_rows    the Newtonian sphere on the same grid (FP64, HLLC, adaptive
               dt found inside the fold vs a separate time-step pass),
               primitive export and CBOR checkpoint rates of the wind state
  cpu_baseline the CPU oracle on this host's cores, bounded sample
`--impl reference` times the CPU implementation of the path (the C++ oracle
port; the reference's Rust crate has no toolchain here) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "app-kilonova_gb300"))

METRIC = "zone-updates/s per GB300: mixed+learned vs plain FP64 GPU at L1<1e-6; HBM %"
UNIT = "zone-updates/s"
# Algorithmic HBM bytes per zone (5 fields, FP64 conserved state): an RK2
# zone-update reads U and writes U1 (80 B), then reads U1 and U0 and writes
# (120 B): 200 B. Geometry counts 0 (recomputable) and halo re-reads are not
# algorithmic. The update launch carries the stage's state traffic, 80 or
# 120 B, on average 100 B per zone. The primitives this design keeps between
# the recovery and the update (FP32, written once and read once per stage:
# 40 B per stage) are an intermediate of the implementation, reported apart.
ALG_BYTES_UPDATE_LAUNCH = 100.0
ACCURACY_STEPS = 200   # the wind workload's configured step count
ALG_BYTES_RECOVERY_LAUNCH = 40.0
ALG_BYTES_PER_ZONE_UPDATE = 200.0
INTERMEDIATE_BYTES_PER_ZONE_UPDATE = 2 * 40.0 + 2 * 20.0 + 2 * 20.0   # U re-read by the recovery, P written and read


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
        # one GPU per rank: the library's contexts use the calling thread's device
        import ctypes as C
        from knc import abi
        lib = abi.load()
        n = C.c_int32()
        if lib.knc_device_count(C.byref(n)) == abi.KNC_OK and n.value > 0:
            lib.knc_set_device(local % n.value)
    return rank, world, local, pg


def barrier(pg):
    if pg:
        pg.barrier()


def max_over_ranks(pg, x: float) -> float:
    if not pg:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def cpu_baseline(workload, blocks: int, steps: int):
    """The CPU oracle on this host's cores: `steps` RK2 steps on `blocks` blocks."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import knc_oracle
    knc_oracle.build()
    threads = os.cpu_count() or 1
    w = workload
    o = knc_oracle.Oracle(w.hydro, w.mesh, threads=threads)
    o.set_model(w.model)
    o.init_from_model(0.0)
    for i in o.block_indexes()[blocks:]:
        o.remove_block(i)
    zones = blocks * w.mesh.block_size * w.mesh.num_polar_zones
    o.advance(1)     # warm caches and page in
    t0 = time.perf_counter()
    o.advance(steps)
    el = time.perf_counter() - t0
    return {"value": zones * steps / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} RK2 steps on {blocks} of {w.num_blocks} blocks ({zones} zones) of the same "
                      f"workload, C++ FP64 oracle, {threads} threads", "seconds": el}


def run_reference(args):
    rank, world, local, pg = dist_setup(args.gpus)
    if rank != 0:
        return 0
    from knc import workloads
    w = workloads.wind_large()
    sys.path.insert(0, str(ROOT / "oracle"))
    import knc_oracle
    knc_oracle.build()
    threads = os.cpu_count() or 1
    blocks = args.ref_blocks
    o = knc_oracle.Oracle(w.hydro, w.mesh, threads=threads)
    o.set_model(w.model)
    o.init_from_model(0.0)
    for i in o.block_indexes()[blocks:]:
        o.remove_block(i)
    zones = blocks * w.mesh.block_size * w.mesh.num_polar_zones
    for _ in range(args.warmup):
        o.advance(1)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.advance(1)
    el = time.perf_counter() - t0
    v = zones * args.steps / el
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": f"{w.name}: wind on 4096x1024 zones, SRHD, PLM 1.5, HLLE, RK2, CFL 0.4; "
                                   f"each step one RK2 step on {blocks} of {w.num_blocks} blocks",
                       "zones_per_step": zones},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"one RK2 step on {blocks} blocks ({zones} zones) per step; the "
                                       "reference's Rust path cannot build here (no cargo/rustc, physics "
                                       "crates not vendored), so this is the C++ oracle restating it"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ncu summaries of the mixed-stage kernels on this workload (one capture each)
# (captured on the strip form of the update, the shape the autotuner picks there)
PROFILE_OF = {"update": "update_strip_mixed_wind_4096x1024.md", "c2p": "c2p_mixed_wind_4096x1024.md"}


def profile_value(name: str, key: str):
    """A `key = value` line of a committed ncu summary under profiles/."""
    f = ROOT / "profiles" / name
    if not f.is_file():
        return None
    for line in f.read_text().splitlines():
        if line.startswith(key + " ") or line.startswith(key + "="):
            return float(line.split("=")[1])
    return None


def profiled_traffic(kernel: str, key: str = "traffic_bytes_per_launch"):
    """DRAM bytes (read + write) of one launch from the committed ncu summary."""
    v = profile_value(PROFILE_OF.get(kernel, ""), key)
    return int(v) if v is not None else None


# FP64 operations per launch of the plain FP64 stage's kernels on this
# workload (DADD + DMUL + 2 DFMA, counted by ncu; data-dependent through the
# Newton iterations, stable for the workload)
FP64_PROFILE = "fp64_kernels_wind_4096x1024.md"


def l1_density(a, b) -> float:
    num = den = 0.0
    for i in b.block_indexes():
        pa = a.get_primitives(i)[..., 0]
        pb = b.get_primitives(i)[..., 0]
        num += float(abs(pa - pb).sum())
        den += float(abs(pb).sum())
    return num / den


def next_rows(args, make, timed, head, w, weights):
    """Measurements of the rows either side of the path (each rank on its own
    GPU; rank 0 reports)."""
    import tempfile
    import numpy as np
    from knc import checkpoint, config, workloads
    out = {}
    # f4 and the Newtonian variant: sphere on 4096 x 1024, HLLC, FP64
    ws = workloads.sphere_large(riemann="HLLC")
    sph = make(False, False, True, workload=ws, tune=True)
    steps, fold = args.next_steps, args.fold
    ms_in, _ = timed(sph, steps, fold)
    # f4 where it matters, folds of one step: dt found in the fold's first
    # recovery (knc_advance) against the reference's order, a full recovery
    # pass for State::time_step and then the step (knc_time_step + knc_advance_dt)
    f4 = {}
    sph.set_batched(False)   # launches issued directly: a one-step graph per call would be re-captured
    for name, sep in (("dt_in_fold", False), ("separate_pass", True)):
        sph.synchronize()
        sph.mark(0)
        for _ in range(args.next_steps // 2):
            if sep:
                sph.advance(1, sph.time_step())
            else:
                sph.advance(1)
        sph.mark(1)
        f4[name + "_ms_per_step"] = sph.elapsed_ms(0, 1) / (args.next_steps // 2)
    out["newtonian_sphere"] = {
        "workload": f"{ws.name}: Newtonian gamma 5/3 seeded density sphere (rho 10 inside r < 2, 1 outside, "
                    "p 1e-2), 4096x1024 zones, HLLC, RK2, CFL 0.4, adaptive dt",
        "path": "FP64, autotuned, CUDA graph per fold", "tuning": sph.tuning(),
        "value": ws.zones * steps / (ms_in * 1e-3), "unit": UNIT, "ms_per_step": ms_in / steps,
        "fold": fold, "steps": steps, "adaptive_dt_fold_of_one": f4}
    sph.close()
    # the reference's own Newtonian flux on the same grid
    wh = workloads.sphere_large(riemann="HLLE")
    sph = make(False, False, True, workload=wh, tune=True)
    ms_h, _ = timed(sph, steps, fold)
    out["newtonian_sphere"]["hlle"] = {"value": wh.zones * steps / (ms_h * 1e-3), "ms_per_step": ms_h / steps,
                                       "tuning": sph.tuning()}
    sph.close()
    # f2: a shipped setup through its device model (setups/jet_in_cloud.yaml:
    # HLLC, 512 polar zones, blocks of 4 radial zones, both excision surfaces
    # moving), mixed + graph against FP64, started at t = 1 as the setup is
    import knc
    from knc import abi
    hydro = config.RelativisticHydro(1.333, 1.5, 0.4, "RK2", "HLLC")
    mesh = config.Mesh(reference_radius=3e8, inner_radius=0.0, outer_radius=0.0, inner_excision_speed=3e8,
                       outer_excision_speed=3e10, num_polar_zones=512, block_size=4)
    model = config.JetInCloud(cloud_mass=1e32, engine_delay=1.0, engine_duration=1.0, engine_strength=1.0,
                              engine_theta=0.1, engine_u=30.0, envelop_m1=2e27, envelop_slowest_beta=0.1,
                              envelop_fastest_beta=0.995, envelop_psi=0.25)
    setup = {"setup": "jet_in_cloud (setups/jet_in_cloud.yaml), device model, start time 1.0"}
    for name, mixed in (("fp64", False), ("mixed_graph", True)):
        sj = knc.Solver(hydro, mesh)
        sj.set_model(model)
        sj.init_from_model(1.0)
        if mixed:
            sj.set_precision(abi.KNC_PRECISION_MIXED)
        sj.set_batched(True)
        sj.autotune(reps=3)
        b0 = len(sj.block_indexes())
        ms_j, _ = timed(sj, steps, fold)
        setup[name] = {"value": timed.zone_updates / (ms_j * 1e-3), "ms_per_step": ms_j / steps,
                       "blocks_start": b0, "blocks_end": len(sj.block_indexes()), "tuning": sj.tuning()}
        sj.close()
    setup["speedup"] = setup["mixed_graph"]["value"] / setup["fp64"]["value"]
    # the learned guess in this setup's FP64 path, where every zone runs the
    # reference's Newton iteration and the relativistic envelope and engine
    # (W up to ~30) need more iterations than a cold wind: plain guess and
    # learned guess on one launch shape, iterations per zone and throughput
    shape = None
    for name, guess in (("fp64_plain_newton", False), ("fp64_learned_guess", True)):
        sj = knc.Solver(hydro, mesh)
        sj.set_model(model)
        sj.init_from_model(1.0)
        if guess:
            sj.set_c2p_guess(abi.KNC_GUESS_MLP, weights)
        sj.set_batched(True)
        if shape is None:
            sj.autotune(reps=3)
            shape = sj.tuning()
        else:
            sj.set_tuning(tile_rows=shape["tile_rows"], fused=shape["fused"], ctas_per_sm=shape["ctas_per_sm"],
                          strip=shape["strip"], deferred=shape["deferred"])
        sj.reset_c2p_stats()
        ms_j, _ = timed(sj, steps, fold)
        st = sj.c2p_stats()
        setup[name] = {"value": timed.zone_updates / (ms_j * 1e-3), "ms_per_step": ms_j / steps,
                       "fp64_iters_per_zone": st["iters_fp64"] / max(st["zones"], 1), "tuning": sj.tuning()}
        sj.close()
    setup["learned_speedup_fp64"] = setup["fp64_learned_guess"]["value"] / setup["fp64_plain_newton"]["value"]
    out["setup_jet_in_cloud"] = setup
    # f3: primitive export of every block of the wind state (device -> host)
    idx = head.block_indexes()
    head.synchronize()
    t0 = time.perf_counter()
    prims = [head.get_primitives(i) for i in idx]
    el = time.perf_counter() - t0
    nbytes = sum(p.nbytes for p in prims)
    out["primitive_export"] = {"blocks": len(idx), "bytes": nbytes, "seconds": el,
                               "GB_per_s": nbytes / el / 1e9}
    # f3 in the reference's own form: a prods.NNNN.cbor file (Products,
    # src/main.rs:51-56) of the wind state, BlockProducts recovered on the device
    ctl_p = config.Control(start_time=0.0, final_time=1.0, checkpoint_interval=0.1, fold=fold)
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "prods.0000.cbor"
        t0 = time.perf_counter()
        checkpoint.write_products(path, head, w.hydro, "wind", {}, w.mesh, ctl_p)
        t_p = time.perf_counter() - t0
        out["products_file"] = {"bytes": path.stat().st_size, "seconds": t_p,
                                "MB_per_s": path.stat().st_size / t_p / 1e6}
    # f1: CBOR checkpoint of the wind state, written and read back (host)
    ctl = config.Control(start_time=0.0, final_time=1.0, checkpoint_interval=0.1, fold=fold)
    with tempfile.TemporaryDirectory() as d:
        path = Path(d) / "chkpt.0000.cbor"
        t0 = time.perf_counter()
        checkpoint.write_checkpoint(path, head, w.hydro, "wind", {}, w.mesh, ctl)
        t_w = time.perf_counter() - t0
        size = path.stat().st_size
        t0 = time.perf_counter()
        ck = checkpoint.read_checkpoint(path)
        t_r = time.perf_counter() - t0
        st = head.state()
        same = all(np.array_equal(ck.blocks[i][0], st[i][0]) and np.array_equal(ck.blocks[i][1], st[i][1])
                   for i in st)
    out["checkpoint"] = {"bytes": size, "write_s": t_w, "read_s": t_r, "write_MB_per_s": size / t_w / 1e6,
                         "read_MB_per_s": size / t_r / 1e6, "round_trip_equal": same,
                         "note": "state download plus CBOR encoding on the host (numpy), one thread"}
    return out


FIELDS = ("D", "S_r", "S_theta", "tau", "scalar_mass")


def field_errors(a, b) -> dict:
    """Per conserved field of solver a against solver b (same blocks):
    relative L1 = sum |a - b| / sum |b| and relative Linf = max |a - b| / max |b|,
    with the momentum magnitude |S| as the scale of both momentum components
    (S_theta of a radial flow is rounding noise around zero)."""
    import numpy as np
    num = np.zeros(5)
    den = np.zeros(5)
    mx = np.zeros(5)
    mb = np.zeros(5)
    for i in b.block_indexes():
        ca, sa = a.get_block(i)
        cb, sb = b.get_block(i)
        smag = np.hypot(cb[..., 1], cb[..., 2])
        for q in range(5):
            x = ca[..., q] if q < 4 else sa
            y = cb[..., q] if q < 4 else sb
            scale = smag if q in (1, 2) else np.abs(y)
            d = np.abs(x - y)
            num[q] += float(d.sum())
            den[q] += float(scale.sum())
            mx[q] = max(mx[q], float(d.max()))
            mb[q] = max(mb[q], float(scale.max()))
    return {FIELDS[q]: {"l1": num[q] / den[q] if den[q] else 0.0, "linf": mx[q] / mb[q] if mb[q] else 0.0}
            for q in range(5)}


def run_knc(args):
    import numpy as np
    import knc
    from knc import abi, learned, workloads

    rank, world, local, pg = dist_setup(args.gpus)
    w = workloads.wind_large(seed=1 + rank)
    zones = w.zones
    hbm_peak, peak_src = load_peaks()

    # ---- learned guess, trained on the device (untimed)
    t0 = time.perf_counter()
    pairs = learned.generate_pairs(w.hydro.gamma_law_index, args.train_pairs, seed=11)
    probe = knc.build_solver(w)
    probe.advance(2)
    run_pairs = learned.sample_pairs(probe, stride=16)
    probe.close()
    all_pairs = np.concatenate([pairs, run_pairs])
    data_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    weights, train_loss = learned.train(all_pairs, steps=args.train_steps, seed=11)
    train_s = time.perf_counter() - t0

    def make(mixed: bool, guess: bool, graph: bool, workload=None, tune=False):
        s = knc.build_solver(workload or w)
        if mixed:
            s.set_precision(abi.KNC_PRECISION_MIXED)
            s.set_mixed_w_split(args.w_split)
        if guess:
            s.set_c2p_guess(abi.KNC_GUESS_MLP, weights)
        s.set_batched(graph)
        if tune:
            s.autotune(reps=3)
        return s

    def timed(s, steps, fold):
        for _ in range(args.warmup):
            s.advance(1)
        s.synchronize()
        barrier(pg)
        l0 = s.launch_count()
        z0 = s.zone_updates()
        s.mark(0)
        done = 0
        while done < steps:
            f = min(fold, steps - done)
            s.advance(f)
            done += f
        s.mark(1)
        ms = s.elapsed_ms(0, 1)
        timed.zone_updates = s.zone_updates() - z0
        return ms, s.launch_count() - l0

    # ---- plain FP64 path
    fp64 = make(False, False, False, tune=True)
    fp64.reset_c2p_stats()
    ms64, _ = timed(fp64, args.steps, args.fold)
    st64 = fp64.c2p_stats()
    ms64 = max_over_ranks(pg, ms64)
    v64 = zones * args.steps * world / (ms64 * 1e-3)
    fp64_peak = knc.measure_fp64_peak()
    # the FP64 kernels timed one after another (CUDA events), against the
    # FP64 FMA rate measured above: this path's own roofline
    p64 = make(False, False, False)
    p64.set_tuning(**fp64.tuning())
    p64.advance(2)
    p64.set_profiling(True)
    p64.advance(4)
    kt64 = p64.kernel_times()
    p64.close()
    fp64_roof = {}
    for kind, key in (("c2p", "flops_per_launch_c2p"), ("update", "flops_per_launch_update")):
        flops = profile_value(FP64_PROFILE, key)
        ms_k = kt64[kind][0] / max(kt64[kind][1], 1)
        if flops and ms_k > 0:
            fp64_roof[kind] = {"ms_per_launch": ms_k, "flops_per_launch": flops,
                               "achieved_gflops": flops / (ms_k * 1e-3) / 1e9,
                               "frac_of_fp64_peak": flops / (ms_k * 1e-3) / 1e9 / fp64_peak}

    # ---- headline: mixed + learned + graph
    clocks = ClockSampler(local)
    head = make(True, True, True, tune=True)
    tuning = head.tuning()
    head.reset_c2p_stats()
    clocks.start()
    msh, launches = timed(head, args.steps, args.fold)
    clk = clocks.stop()
    sth = head.c2p_stats()
    msh = max_over_ranks(pg, msh)
    value = zones * args.steps * world / (msh * 1e-3)
    l1_run = l1_density(head, fp64)   # after this run's warm-up + timed steps
    # the accuracy gate at the workload's own step count (200 RK2 steps),
    # whatever --steps this run timed: a fresh pair of solvers
    # (and again after twice as many steps, how the error grows)
    acc_m, acc_64 = make(True, True, True), make(False, False, True)
    acc_m.set_tuning(**tuning)

    def advance_both(n):
        for s_ in (acc_m, acc_64):
            for _ in range(n // args.fold):
                s_.advance(args.fold)
            if n % args.fold:
                s_.advance(n % args.fold)

    advance_both(ACCURACY_STEPS)
    l1 = l1_density(acc_m, acc_64)
    errs = field_errors(acc_m, acc_64)
    acc_steps = ACCURACY_STEPS
    advance_both(ACCURACY_STEPS)
    l1_twice = l1_density(acc_m, acc_64)
    acc_m.close()
    acc_64.close()

    # ---- same path without the graph, kernels timed with events (roofline)
    prof = make(True, True, False)
    prof.set_tuning(**tuning)
    for _ in range(args.warmup):
        prof.advance(1)
    prof.set_profiling(True)
    prof.advance(args.steps)
    kt = prof.kernel_times()
    prof.set_profiling(False)
    prof.close()
    dom = max(kt, key=lambda k: kt[k][0])
    dom_ms = kt[dom][0] / max(kt[dom][1], 1)
    # one launch processes one stage of every zone
    per_zone = {"update": ALG_BYTES_UPDATE_LAUNCH, "c2p": ALG_BYTES_RECOVERY_LAUNCH}.get(dom, 0.0)
    alg_bytes = per_zone * zones
    achieved = alg_bytes / (dom_ms * 1e-3) / 1e9
    traffic = profiled_traffic(dom) if (dom != "update" or tuning.get("strip")) else None
    # per stage, against that stage's algorithmic bytes (the update launch:
    # stage 1 reads U and writes U1, 80 B per zone; stage 2 reads U1 and U0
    # and writes the average, 120 B)
    per_stage = None
    if dom == "update" and tuning.get("strip"):
        per_stage = {}
        for k, alg in ((1, 80.0), (2, 120.0)):
            t = profiled_traffic("update", f"traffic_bytes_stage{k}")
            if t:
                per_stage[f"stage{k}"] = {"alg_bytes": alg * zones, "traffic": t, "ratio": t / (alg * zones)}

    # ---- end to end through the C ABI with host buffers
    nb = w.num_blocks
    cons = knc.solver.PinnedArray((nb, w.mesh.block_size, w.mesh.num_polar_zones, 4))
    scal = knc.solver.PinnedArray((nb, w.mesh.block_size, w.mesh.num_polar_zones))
    head.get_state(cons.array, scal.array)
    for _ in range(args.warmup):
        head.advance_host(cons.array, scal.array, 1)
    barrier(pg)
    head.mark(2)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        head.advance_host(cons.array, scal.array, 1)
    wall = time.perf_counter() - t0
    head.mark(3)
    e2e_ms = max_over_ranks(pg, max(head.elapsed_ms(2, 3), wall * 1e3))
    e2e = zones * args.steps * world / (e2e_ms * 1e-3)
    h2d = cons.array.nbytes + scal.array.nbytes

    # ---- batched uneven blocks with moving excision (RK3, autotuned launch shape)
    un = None
    if not args.no_uneven:
        wu = workloads.uneven(seed=1 + rank)
        u64 = make(False, False, False, workload=wu, tune=True)
        ms_u64, _ = timed(u64, args.steps, args.fold)
        zu64 = timed.zone_updates
        ms_u64 = max_over_ranks(pg, ms_u64)

        def run_c4(tuning=None):
            """The mixed + learned + graph path on the uneven workload with the
            autotuner's launch shape (tuning None) or the given one."""
            s = make(True, True, True, workload=wu, tune=tuning is None)
            if tuning is not None:
                s.set_tuning(**tuning)
            ms, launches = timed(s, args.steps, args.fold)
            z = timed.zone_updates
            ms = max_over_ranks(pg, ms)
            r = {"value": z * world / (ms * 1e-3), "ms_per_step": ms / args.steps,
                 "launches_per_stage": launches / (3 * args.steps), "tuning": s.tuning(),
                 "blocks_end": len(s.block_indexes()),
                 "block_range_end": [s.block_indexes()[0], s.block_indexes()[-1]],
                 "speedup_vs_fp64": (z / ms) / (zu64 / ms_u64),
                 "l1_density": l1_density(s, u64) if s.block_indexes() == u64.block_indexes() else None}
            s.close()
            return r

        auto = run_c4()
        t = auto["tuning"]
        rows = t["tile_rows"] if t["strip"] else 16
        # the autotuner times single stages launched from the host; the timed
        # run replays captured folds, where launch gaps are hidden, so the
        # other family of shapes is timed the same way too: the separate
        # deferring launches, or every RK3 stage as one cooperative launch (the
        # fused deferring form with one 20-warp CTA per SM, or 4 or 5 4-warp
        # CTAs per SM)
        fused = auto if t["fused"] else None
        separate = None if t["fused"] else auto
        if fused is None:
            for k in (1, 4, 5):
                r = run_c4(dict(tile_rows=rows, fused=True, strip=True, ctas_per_sm=k, deferred=True))
                if fused is None or r["ms_per_step"] < fused["ms_per_step"]:
                    fused = r
        else:
            separate = run_c4(dict(tile_rows=rows, strip=True, ctas_per_sm=5, deferred=True))
        best = fused if fused["ms_per_step"] < separate["ms_per_step"] else separate
        un = {"workload": f"{wu.name}: {wu.zones} zones at start, nr from 32..512 and nq from 64..256 "
                          "per block (seeded), RK3, both excision surfaces at 0.5c",
              "zones_start": wu.zones, "blocks_end": best["blocks_end"],
              "block_range_end": best["block_range_end"],
              "value": best["value"], "fp64_value": zu64 * world / (ms_u64 * 1e-3),
              "speedup_vs_fp64": best["speedup_vs_fp64"],
              "ms_per_step": best["ms_per_step"], "fp64_ms_per_step": ms_u64 / args.steps,
              "l1_density": best["l1_density"], "tuning": best["tuning"],
              "launches_per_stage": best["launches_per_stage"],
              "autotuned_tuning": t,
              "separate_launches": separate, "one_launch_per_stage": fused,
              "path": "mixed + learned guess + one CUDA graph per fold; the faster of the separate launches and "
                      "the one-launch-per-stage form, both timed as captured folds"}
        u64.close()

    # ---- the learned guess inside the W = 100 jet (2048 x 512), against plain
    # Newton from the reference's guess: FP64 / FP32 iterations per zone and
    # throughput, each path on its autotuned shape, density L1 against FP64
    jet = None
    if not args.no_jet:
        wj = workloads.jet(seed=1 + rank)
        # the jet's configured step count in all (warm-up steps included), so
        # the density L1 is the accuracy gate at that count
        jet_steps = args.jet_steps if args.jet_steps else wj.steps - args.warmup
        j64 = make(False, False, False, workload=wj)
        timed(j64, jet_steps, args.fold)
        jet = {"workload": f"{wj.name}: relativistic jet, W = 100, theta_j = 0.1, p/rho = 1e-3, through r = 1 "
                           "into a seeded r^-2 ambient, 2048x512 zones in 32 blocks of 64x512, RK2",
               "zones": wj.zones, "steps": jet_steps, "accuracy_steps": jet_steps + args.warmup,
               "mixed_faces": f"FP64 where the stencil reaches a zone above W = {args.w_split}, else FP32"}
        # each pair (plain / learned guess) on one launch shape, the one the
        # autotuner picks for the plain guess, so the pair differs in the guess only
        shape = {}
        for name, guess, mixed in (("plain_newton", False, True), ("learned_guess", True, True),
                                   ("fp64_plain_newton", False, False), ("fp64_learned_guess", True, False)):
            sj = make(mixed, guess, True, workload=wj, tune=mixed not in shape)
            if mixed in shape:
                t = shape[mixed]
                sj.set_tuning(tile_rows=t["tile_rows"], fused=t["fused"], ctas_per_sm=t["ctas_per_sm"],
                              tma=t["tma"], strip=t["strip"], deferred=t["deferred"])
            else:
                shape[mixed] = sj.tuning()
            sj.reset_c2p_stats()
            ms_j, _ = timed(sj, jet_steps, args.fold)
            ms_j = max_over_ranks(pg, ms_j)
            st = sj.c2p_stats()
            jet[name] = {"value": wj.zones * jet_steps * world / (ms_j * 1e-3),
                         "ms_per_step": ms_j / jet_steps,
                         "fp64_iters_per_zone": st["iters_fp64"] / max(st["zones"], 1),
                         "fp32_iters_per_zone": st["iters_fp32"] / max(st["zones"], 1),
                         "fallbacks": st["fallbacks"], "l1_density": l1_density(sj, j64),
                         "errors_vs_fp64": field_errors(sj, j64) if mixed else None,
                         "tuning": sj.tuning()}
            sj.close()
        j64.close()
        # FP64 Newton iterations the learned start saves: in the mixed path
        # (FP64 only for the zones above the split, started from the FP32
        # root) and in the FP64 path (every zone, reference iteration)
        for key, a_, b_ in (("fp64_iters_saved_mixed", "learned_guess", "plain_newton"),
                            ("fp64_iters_saved_fp64_path", "fp64_learned_guess", "fp64_plain_newton")):
            jet[key] = 1.0 - jet[a_]["fp64_iters_per_zone"] / max(jet[b_]["fp64_iters_per_zone"], 1e-30)

    # ---- the rows around the path: the Newtonian sphere of the same grid
    # (FP64, HLLC, adaptive dt found inside the fold) against the separate
    # time-step pass, primitive export and CBOR checkpoints of the wind state
    nxt = None
    if not args.no_next:
        # every rank (its own replica): the timed loops hold a barrier
        nxt = next_rows(args, make, timed, head, w, weights)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(w, args.cpu_blocks, args.cpu_steps)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": msh / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 state+recovery / f32 flux",
            "data": "synthetic",
            "config": {"workload": f"{w.name}: relativistic wind, 4096x1024 zones in 64 blocks of 64x1024, "
                                   "gamma 4/3, PLM theta 1.5, HLLE, RK2, CFL 0.4",
                       "zones": zones, "path": f"mixed precision (FP64 recovery above W={args.w_split}), "
                                               "learned c2p guess, CUDA graph per fold",
                       "fold": args.fold, "l2": "state 168 MB per buffer > 129 MB L2 (no flush needed)",
                       "parallelism": f"replicas x{world}", "tuning": tuning},
            "fp64": {"value": v64, "ms_per_step": ms64 / args.steps, "tuning": fp64.tuning(),
                     "newton_iters_per_zone": st64["iters_fp64"] / max(st64["zones"], 1),
                     "fp64_peak_gflops": fp64_peak, "fp64_roofline": fp64_roof},
            "speedup_vs_fp64": value / v64,
            "l1_density": l1,
            "errors_vs_fp64": errs,
            "accuracy_steps": acc_steps,
            "l1_density_twice_the_steps": l1_twice,
            "l1_density_after_run": l1_run,
            "c2p": {"fp64_iters_per_zone": sth["iters_fp64"] / max(sth["zones"], 1),
                    "fp32_iters_per_zone": sth["iters_fp32"] / max(sth["zones"], 1),
                    "fallbacks": sth["fallbacks"], "mlp_train_loss": train_loss, "mlp_train_s": train_s,
                    "mlp_train_steps": args.train_steps, "mlp_train_pairs": len(all_pairs), "mlp_data_s": data_s},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                         "peak_source": peak_src, "avg_launch_ms": dom_ms,
                         "traffic_ratio": traffic / alg_bytes if traffic else None,
                         "traffic_per_stage": per_stage,
                         "kernel_ms": {k: v[0] / max(v[1], 1) for k, v in kt.items()},
                         "alg_bytes_per_zone_launch": per_zone,
                         "step": {"alg_bytes_per_zone_update": ALG_BYTES_PER_ZONE_UPDATE,
                                  "achieved": ALG_BYTES_PER_ZONE_UPDATE * value / 1e9,
                                  "frac": ALG_BYTES_PER_ZONE_UPDATE * value / 1e9 / hbm_peak,
                                  "with_intermediates_frac": (ALG_BYTES_PER_ZONE_UPDATE +
                                                              INTERMEDIATE_BYTES_PER_ZONE_UPDATE) * value / 1e9 /
                                                             hbm_peak}},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d},
            "gpu_launches": launches,
            "clocks": clk,
        }
        if un:
            line["batched_uneven"] = un
        if jet:
            line["learned_jet"] = jet
        if nxt:
            line["next_rows"] = nxt
        if cpu:
            line["cpu_baseline"] = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
        print(json.dumps(line), flush=True)
    if pg:
        pg.destroy_process_group()
    return 0


def run_only(args):
    """One path alone on the workload, for profiler captures: warmup + steps."""
    import knc
    from knc import abi, learned, workloads
    w = workloads.WORKLOADS[args.workload]()
    s = knc.build_solver(w)
    if args.tile_rows:
        s.set_tuning(tile_rows=args.tile_rows, fused=args.fused, tma=args.tma, strip=args.strip,
                     ctas_per_sm=args.ctas_per_sm, deferred=args.deferred)
    if args.only == "mixed":
        s.set_precision(abi.KNC_PRECISION_MIXED)
        s.set_mixed_w_split(args.w_split)
        if args.train_steps > 0:
            pairs = learned.generate_pairs(w.hydro.gamma_law_index, args.train_pairs, seed=11)
            weights, _ = learned.train(pairs, steps=args.train_steps, seed=11)
            s.set_c2p_guess(abi.KNC_GUESS_MLP, weights)
    for _ in range(args.warmup):
        s.advance(1)
    s.mark(0)
    s.advance(args.steps)
    s.mark(1)
    ms = s.elapsed_ms(0, 1)
    print(json.dumps({"only": args.only, "zones": w.zones, "steps": args.steps,
                      "value": w.zones * args.steps / (ms * 1e-3), "ms_per_step": ms / args.steps}), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="knc", choices=["knc", "reference"])
    ap.add_argument("--fold", type=int, default=50)
    ap.add_argument("--w-split", type=float, default=2.0)
    ap.add_argument("--train-pairs", type=int, default=10_000_000)
    ap.add_argument("--train-steps", type=int, default=3000)
    ap.add_argument("--cpu-blocks", type=int, default=16)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--ref-blocks", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-uneven", action="store_true")
    ap.add_argument("--no-jet", action="store_true")
    ap.add_argument("--no-next", action="store_true")
    ap.add_argument("--next-steps", type=int, default=50)
    ap.add_argument("--jet-steps", type=int, default=0, help="0: the jet's configured steps less the warm-up")
    ap.add_argument("--workload", default="wind_large", help="workload of --only runs")
    ap.add_argument("--tile-rows", type=int, default=0, help="launch shape of --only runs (0: default)")
    ap.add_argument("--fused", action="store_true")
    ap.add_argument("--tma", action="store_true")
    ap.add_argument("--strip", action="store_true")
    ap.add_argument("--ctas-per-sm", type=int, default=0)
    ap.add_argument("--deferred", action="store_true", help="mixed recovery with the FP64 zones deferred")
    ap.add_argument("--only", choices=["fp64", "mixed"], default=None,
                    help="run one path alone (profiler captures)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.only:
        return run_only(args)
    return run_knc(args)


if __name__ == "__main__":
    sys.exit(main())
