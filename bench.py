#!/usr/bin/env python3
"""Benchmark of the GB300 CVF engine: site-updates/ns on the L=256 checkerboard workload.

Workload (one "step"): one cube (eta) move, one NPT volume move and one checkerboard Metropolis
sweep of an L=256 lattice (16,777,216 cells, one uint32 per cell = 64 MB), ordered start,
T=0.70, P=0.45, Metropolis only -- the bandwidth-bound single-lattice configuration.
site-updates/ns counts a cell (all six sigma arms attempted) as one site update.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl engine|reference]
                  [--workload l256|batch64]

Timing: W untimed warm-up steps, then K steps each bracketed by CUDA events on the engine's own
stream; the 64 MB lattice fits in the 129 MB L2, so a 256 MB buffer is written on the same
stream before every timed step (outside the events). Under torchrun every rank steps its own
replica (independent lattices, no collective); rank 0 prints the whole-job line.
--impl reference times the CPU oracle (the reference's CPU path does not compile, so the
restatement in oracle/ stands in) on all host cores, rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L_BENCH, T_BENCH, P_BENCH, SEED = 256, 0.70, 0.45, 44648604
ALG_BYTES_PER_CELL_SWEEP = 8  # read + write one packed uint32 per cell per sweep


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_params(rank, local=0):
    """The lattice rank `rank` steps: the L=256 workload with its own seed and replica id, so the
    ranks' chains are independent and need no collective (weak scaling, replicas only)."""
    from cvfbulkwater_gb300.engine import Params
    return Params(L=L_BENCH, T=T_BENCH, P=P_BENCH, seed=SEED + rank, start=2, replica=rank, device=local)


class Dist:
    """Barrier and max-over-ranks on a CPU (gloo) group; a no-op for one process."""

    def __init__(self, world):
        self.world = world
        if world > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
            self.td = td

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class NvmlClocks:
    """Reads SM clocks and clock-event reasons through NVML (libnvidia-ml, read-only queries) from
    a thread every 2 ms while the timed region runs; None when NVML cannot be loaded."""

    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown", 0x4: "sw_power_cap"}

    def __init__(self, gpu: int):
        import ctypes as C
        import threading
        self.C, self.threading = C, threading
        self.lib = C.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = C.c_void_p()
        if self.lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(gpu), C.byref(self.h)) != 0:
            raise OSError("no NVML handle")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        self.rows, self.stop_flag, self.thread = [], False, None

    def _sample(self):
        C = self.C
        mhz, mx, rs = C.c_uint(), C.c_uint(), C.c_ulonglong()
        while not self.stop_flag:
            if (self.lib.nvmlDeviceGetClockInfo(self.h, 1, C.byref(mhz)) == 0 and
                    self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(mx)) == 0 and
                    self.reasons_fn(self.h, C.byref(rs)) == 0):
                self.rows.append((mhz.value, mx.value, rs.value))
            time.sleep(0.002)

    def start(self):
        self.thread = self.threading.Thread(target=self._sample, daemon=True)
        self.thread.start()

    def stop(self):
        self.stop_flag = True
        self.thread.join(timeout=5)
        try:
            self.lib.nvmlShutdown()
        except Exception:
            pass
        if not self.rows:
            return None
        reasons = sorted({n for _, _, r in self.rows for b, n in self.REASONS.items() if r & b})
        return {"sm_mhz": float(np.median([r[0] for r in self.rows])), "sm_max_mhz": float(max(r[1] for r in self.rows)),
                "reasons": reasons, "samples": len(self.rows), "source": "NVML, every 2 ms"}


class Clocks:
    """Samples SM clocks and throttle reasons while the timed region runs: through NVML when the
    library loads, else with nvidia-smi."""

    def __new__(cls, gpu: int):
        try:
            return NvmlClocks(gpu)
        except (OSError, AttributeError):
            return super().__new__(cls)

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None
        self.skip = 0

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        # the sampler takes a moment to start: wait (at most 3 s) for its first line, so that the
        # timed region that follows is sampled from its start
        t0 = time.time()
        while time.time() - t0 < 3.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)
        with open(self.path) as f:
            self.skip = sum(1 for _ in f)  # lines written before the timed region

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if len(rows) > self.skip:
            rows = rows[self.skip:]  # the samples taken while the timed region ran
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": float(np.median([r[0] for r in rows])), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(name, tile=None):
    """DRAM bytes per launch from a committed ncu summary under profiles/ (the entry of the sweep
    tile when the summary has one per tile), if there is one."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    try:
        d = json.load(open(p))
    except (ValueError, OSError):
        return None
    if tile is not None and "by_tile" in d:
        return d["by_tile"].get(str(tile), {}).get("dram_bytes_per_launch")
    return d.get("dram_bytes_per_launch")


def issue_roof(tile, cells_per_launch, launch_s, sm_mhz, n_sm):
    """Instruction-issue roofline of the sweep launch: thread instructions per cell (from the
    committed ncu summary of the same kernel and tile) x cells per launch / launch time, against
    the issue peak of the SMs (4 schedulers x 32 lanes per SM per cycle) at the sampled clock."""
    p = os.path.join(ROOT, "profiles", "sweep_l256_issue.json")
    if not os.path.exists(p):
        return None
    try:
        per_cell = json.load(open(p))["by_tile"][str(tile)]["thread_inst_per_cell"]
    except (ValueError, OSError, KeyError):
        return None
    achieved = per_cell * cells_per_launch / launch_s
    peak = n_sm * 4 * 32 * sm_mhz * 1e6
    return {"thread_inst_per_cell": per_cell, "achieved": round(achieved / 1e12, 3),
            "peak": round(peak / 1e12, 3), "unit": "T thread-instructions/s", "frac": round(achieved / peak, 4),
            "sm_mhz": sm_mhz, "source": "profiles/sweep_l256_issue.json"}


def cpu_baseline_oracle(steps_cap=3, budget_s=30.0, threads=None):
    """The CPU oracle on all host cores (or `threads`) over a bounded sample of the same workload."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    o = O.Oracle(L_BENCH, T_BENCH, P_BENCH, SEED, 6.0, 0, 2, threads=threads)
    o.step(1, 0)  # warm-up
    t0 = time.perf_counter()
    n = 0
    while n < steps_cap and (time.perf_counter() - t0) < budget_s:
        o.step(1, 0)
        n += 1
    dt = time.perf_counter() - t0
    o.close()
    val = L_BENCH ** 3 * n / dt / 1e9
    return {"value": round(val, 6), "unit": "site-updates/ns", "cores": threads, "kind": "port",
            "sample": f"{n} full MC steps (cube + volume + sweep) of the L=256 lattice on {threads} "
                      f"OpenMP threads ({dt:.1f} s)"}


def warm_steps(lat, n, nmet=1, ncl=0):
    """n (at least 3) untimed steps as the timed loops make them, one run call per step, so the
    one-step graph is built and warm before the timed region."""
    for _ in range(max(3, n)):
        lat.run(1, nmet, ncl)
    lat.synchronize()


def timed_steps(lat, steps, flush, nmet=1, ncl=0):
    """Device time (ms) of `steps` MC steps of a handle, each bracketed by CUDA events on the
    handle's stream with a 256 MB L2 flush before it."""
    import torch
    stream = torch.cuda.ExternalStream(lat.stream_ptr())
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for i in range(steps):
            flush.fill_(i & 255)
            ev[i][0].record(stream)
            lat.run(1, nmet, ncl)
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in ev)


def batch_params(local):
    """Batched workload: 64 replicas, L drawn from {16,24,32,48,64} with a fixed seed, on the 8x8
    grid T in [0.55, 0.95] x P in [0.0, 0.60], disordered starts from per-replica seeds."""
    from cvfbulkwater_gb300.engine import Params
    rng = np.random.default_rng(20261203)
    Ls = rng.choice([16, 24, 32, 48, 64], size=64)
    Ts = np.linspace(0.55, 0.95, 8)
    Ps = np.linspace(0.0, 0.60, 8)
    return [Params(L=int(Ls[i]), T=float(Ts[i % 8]), P=float(Ps[i // 8]), seed=SEED + i, start=0, replica=i,
                   device=local) for i in range(64)]


def bench_batch64(steps, warmup, local, flush, verify=4):
    """One batched handle (one set of launches per step for all 64 replicas, graph-captured,
    autotuned tile) against the same 64 replicas run one after another as plain handles. The
    chains are identical (same Philox streams), so "equal error" holds sample for sample; the
    first `verify` replicas are compared bit for bit."""
    from cvfbulkwater_gb300.engine import Lattice
    params = batch_params(local)
    cells = sum(p.L ** 3 for p in params)
    batch = Lattice(params)
    tile = batch.autotune()
    tuned = batch.tuning()
    warm_steps(batch, warmup)
    t_batch = timed_steps(batch, steps, flush)
    t_plain = 0.0
    same = True
    for i, p in enumerate(params):
        h = Lattice(p)
        warm_steps(h, warmup)
        t_plain += timed_steps(h, steps, flush)
        if i < verify:
            same = same and bool(np.array_equal(h.get_config(), batch.get_config(i)))
        h.close()
    batch.close()
    rs_b = 64 * steps / (t_batch / 1e3)
    rs_p = 64 * steps / (t_plain / 1e3)
    return {"workload": "64 replicas, L from {16,24,32,48,64} (seeded), 8x8 grid T 0.55..0.95 x P 0..0.60, "
                        "disordered starts; 1 cube + 1 volume move + 1 sweep per step",
            "cells": cells, "steps": steps, "sweep_tile": tile, "tuning": dict(zip(("tile", "lg_rows", "launch_mode"), tuned)),
            "batched_replica_sweeps_per_s": round(rs_b, 1),
            "plain_sequential_replica_sweeps_per_s": round(rs_p, 1),
            "batched_site_updates_per_ns": round(cells * steps / (t_batch * 1e6), 4),
            "plain_site_updates_per_ns": round(cells * steps / (t_plain * 1e6), 4),
            "speedup": round(t_plain / t_batch, 2), "identical_chains_checked": verify, "identical": same,
            "l2": "256 MB write before every timed step in both arms", "occupancy": batch_occupancy()}


def batch_occupancy():
    """SM occupancy of the batch's kernels (achieved and theoretical warps per SM, waves) from the
    committed ncu summary of the same workload; None where the summary is absent."""
    p = os.path.join(ROOT, "profiles", "batch64_occupancy.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    return dict(d["summary"], source="profiles/batch64_occupancy.json")


def sample_columns(lat, smp, r=0):
    """E, V and N_hb of every record from the sample fields, vectorised with the engine's own
    formulas (GW:2014-2160; E_vdW summed over the shells in their order, each operation rounded
    as in the library)."""
    d, f = lat.get_distances(r)
    Rc = float(np.float32(6.0))
    rr = smp["r_cell"].astype(np.float64)
    t = 1.0 / Rc
    t = t * t * t
    att = t * t
    shift = att * att - att
    ev = np.zeros_like(rr)
    for di, fi in zip(d.astype(np.float64), f.astype(np.float64)):
        rd = rr * di
        m = rd < Rc
        tmp = np.where(m, 1.0 / np.where(m, rd, 1.0), 0.0)
        tmp = tmp * tmp * tmp
        a = tmp * tmp
        ev = np.where(m, ev + fi * ((a * a - a) - shift), ev)
    nhb = smp["n_hb2"].astype(np.float64) * 0.5
    e = (ev + (-float(np.float32(0.5))) * nhb) + (-float(np.float32(0.08))) * smp["n_sigma"].astype(np.float64)
    v = smp["volume"].astype(np.float64) + float(np.float32(0.6)) * nhb
    return e, v, nhb


def bench_differentiation(local):
    """Differentiable reweighting workload: 32 replicas of L=32 along P=0.45 at T uniform
    in [0.60, 0.90], 100,000 recorded steps each (3.2 M samples); FP64 WHAM forward and adjoint;
    alpha_P, K_T, C_P at T = 0.75 from the adjoint against finite differences and the fluctuation
    formulas; the reweighted density against the reference's L32 P=0.45 isobar."""
    import ctypes as C
    from cvfbulkwater_gb300 import abi
    from cvfbulkwater_gb300.engine import Lattice, Params
    L, N, P0, R, K = 32, 32 ** 3, 0.45, 32, 100000
    temps = np.linspace(0.60, 0.90, R)
    # five more runs for the finite differences of independent runs: (0.75, P0) and its neighbours
    # at T +/- 0.005 and P +/- 0.005, the same sampling
    fd_pts = [(0.75, P0), (0.745, P0), (0.755, P0), (0.75, P0 - 0.005), (0.75, P0 + 0.005)]
    lat = Lattice([Params(L=L, T=float(t), P=P0, seed=SEED + 500 + i, start=0, replica=i, device=local,
                          sample_capacity=K) for i, t in enumerate(temps)] +
                  [Params(L=L, T=t, P=p, seed=SEED + 600 + i, start=0, replica=R + i, device=local, sample_capacity=K)
                   for i, (t, p) in enumerate(fd_pts)])
    lat.run(3000, 1, 0)
    lat.synchronize()
    t0 = time.perf_counter()
    lat.run_sampled(K, 1, 0, 1)
    lat.synchronize()
    t_sample = time.perf_counter() - t0
    cols, run_of = [], []
    for r in range(R):
        smp = lat.samples(r)
        e, v, nhb = sample_columns(lat, smp, r)
        cols.append(np.stack([e, v, nhb, smp["n_sigma"].astype(np.float64)], axis=1))
        run_of.append(np.full(len(smp), r, dtype=np.int32))
    fd_runs = []
    for i, (t, p) in enumerate(fd_pts):
        smp = lat.samples(R + i)
        e, v, nhb = sample_columns(lat, smp, R + i)
        fd_runs.append({"E": e, "V": v, "H": e + float(np.float32(p)) * v})
    lat.close()
    s = np.ascontiguousarray(np.concatenate(cols))
    ro = np.ascontiguousarray(np.concatenate(run_of))
    runs = np.ascontiguousarray([[1.0 / float(np.float32(t)), float(np.float32(P0))] for t in temps])
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    ids = {"E": 0, "V": 1, "NHB": 2, "NSIG": 3, "H": 4, "RHO": 5, "H2": 6, "V2": 7, "VH": 8}

    def forward(theta, obs, f, n_iter):
        o = np.ascontiguousarray([ids[k] for k in obs], dtype=np.int32)
        out = np.zeros(len(obs) + 1)
        th = np.ascontiguousarray(theta, dtype=np.float64)
        abi.check(abi.lib().cvf_reweight_forward(local, ptr(s), ptr(ro), len(s), ptr(runs), R, ptr(f), n_iter, 1e-10,
                                                 float(N), ptr(th), ptr(o), len(obs), ptr(out)))
        return out[:-1]

    def adjoint(theta, obs, f, g):
        o = np.ascontiguousarray([ids[k] for k in obs], dtype=np.int32)
        th = np.ascontiguousarray(theta, dtype=np.float64)
        gg = np.ascontiguousarray(g, dtype=np.float64)
        out = np.zeros(5)
        abi.check(abi.lib().cvf_reweight_adjoint(local, ptr(s), ptr(ro), len(s), ptr(runs), R, ptr(f), float(N),
                                                 ptr(th), ptr(o), len(obs), ptr(gg), ptr(out)))
        return out

    P = float(np.float32(P0))
    th = lambda t, p=P: [1.0 / t, p, 0.0, 0.0, 0.0]  # noqa: E731
    f = np.zeros(R)
    n_it = 200
    t0 = time.perf_counter()
    forward(th(0.75), ["V"], f, n_it)
    t_wham = time.perf_counter() - t0
    f_next = f.copy()
    forward(th(0.75), ["V"], f_next, 1)
    wham_change = float(np.max(np.abs(f_next - f)))
    t0 = time.perf_counter()
    V, H, V2, H2, VH = forward(th(0.75), ["V", "H", "V2", "H2", "VH"], f, 0)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    gV = adjoint(th(0.75), ["V"], f, [1.0])
    t_adj = time.perf_counter() - t0
    gH = adjoint(th(0.75), ["H"], f, [1.0])
    t = 0.75
    ap_adj = -gV[0] / (t * t) / V  # d/dT = -beta^2 d/dbeta
    kt_adj = -gV[1] / V
    cp_adj = -gH[0] / (t * t) / N
    vp, vm = forward(th(0.755), ["V"], f, 0)[0], forward(th(0.745), ["V"], f, 0)[0]
    hp, hm = forward(th(0.755), ["H"], f, 0)[0], forward(th(0.745), ["H"], f, 0)[0]
    vpp, vpm = forward(th(0.75, P + 0.005), ["V"], f, 0)[0], forward(th(0.75, P - 0.005), ["V"], f, 0)[0]
    independent = independent_run_check(fd_runs, fd_pts, N, {"alpha_P": ap_adj, "K_T": kt_adj, "C_P": cp_adj})
    gold = {round(a, 3): (b, c) for a, b, c in np.loadtxt(os.path.join(ROOT, "tests", "golden", "isobar_P0.45_density.txt"))}
    cmp = []
    for tt in sorted(k for k in gold if 0.6 <= k <= 0.9):
        rho = forward(th(tt), ["RHO"], f, 0)[0]
        want, err = gold[tt]
        cmp.append([tt, round(float(rho), 6), want, round(float((rho - want) / err), 2)])
    return {"workload": f"{R} replicas, L={L}, P=0.45, T uniform in [0.60, 0.90], {K} recorded steps each "
                        f"({len(s)} samples, {len(s) * 32 / 1e6:.0f} MB of records on the device)",
            "sampling_s": round(t_sample, 3),
            "sampling_site_updates_per_ns": round(R * N * K / t_sample / 1e9, 2),
            "wham_ms_per_iteration": round(t_wham / n_it * 1e3, 3),
            "wham_last_change": wham_change,
            "fp64_exp_per_s_in_wham": round(len(s) * R * n_it / t_wham / 1e9, 2),
            "forward_ms": round(t_fwd * 1e3, 3), "adjoint_ms": round(t_adj * 1e3, 3),
            "response_T0.75": {
                "alpha_P": {"adjoint": ap_adj, "finite_difference": (vp - vm) / 0.01 / V,
                            "fluctuation": (VH - V * H) / (t * t * V)},
                "K_T": {"adjoint": kt_adj, "finite_difference": -(vpp - vpm) / 0.01 / V,
                        "fluctuation": (V2 - V * V) / (t * V)},
                "C_P": {"adjoint": cp_adj, "finite_difference": (hp - hm) / 0.01 / N,
                        "fluctuation": (H2 - H * H) / (t * t * N)}},
            "response_vs_independent_runs": independent,
            "rho_vs_reference_isobar": {"columns": ["T", "reweighted", "reference", "(rw - ref) / ref_err"],
                                        "rows": cmp}}


def independent_run_check(runs, pts, N, reweighted, nb=20):
    """alpha_P, K_T and C_P from central differences of the means of independent runs at T0 +/-
    0.005 and P0 +/- 0.005 (20-block errors; the finite differences of the reference's
    CVF_ThermodynamicAnalysis programs), against the adjoint's fluctuation formulas on the run at
    (T0, P0) itself (jackknife errors over the same blocks) and the adjoint of the reweighted
    32-run ensemble at (T0, P0): z = (adjoint - difference) / combined error."""
    def blocks(x):
        x = np.asarray(x)[: len(x) // nb * nb]
        return x.reshape(nb, -1)

    def mean_err(x):
        b = blocks(x).mean(1)
        return float(b.mean()), float(b.std(ddof=1) / np.sqrt(nb))

    def jack(f, *cols):
        bl = [blocks(c) for c in cols]
        v = np.array([f(*[np.delete(b, k, axis=0).ravel() for b in bl]) for k in range(nb)])
        return float(np.sqrt((nb - 1) / nb * ((v - v.mean()) ** 2).sum()))

    Tf = [float(np.float32(t)) for t, _ in pts]
    Pf = [float(np.float32(p)) for _, p in pts]
    dT, dP = Tf[2] - Tf[1], Pf[4] - Pf[3]
    beta = 1.0 / Tf[0]
    c = runs[0]
    V0 = float(c["V"].mean())
    (hm, ehm), (hp, ehp) = mean_err(runs[1]["H"]), mean_err(runs[2]["H"])
    (vm, evm), (vp, evp) = mean_err(runs[1]["V"]), mean_err(runs[2]["V"])
    (wm, ewm), (wp, ewp) = mean_err(runs[3]["V"]), mean_err(runs[4]["V"])
    fd = {"C_P": ((hp - hm) / dT / N, float(np.hypot(ehp, ehm)) / dT / N),
          "alpha_P": ((vp - vm) / dT / V0, float(np.hypot(evp, evm)) / dT / V0),
          "K_T": (-(wp - wm) / dP / V0, float(np.hypot(ewp, ewm)) / dP / V0)}
    fl = {"C_P": (lambda h: beta * beta * h.var() / N, (c["H"],)),
          "alpha_P": (lambda v, h: beta * beta * float(np.mean((v - v.mean()) * (h - h.mean()))) / v.mean(),
                      (c["V"], c["H"])),
          "K_T": (lambda v: beta * v.var() / v.mean(), (c["V"],))}
    out = {}
    for k in ("alpha_P", "K_T", "C_P"):
        f, cols = fl[k]
        val, err = f(*cols), jack(f, *cols)
        d, e = fd[k]
        out[k] = {"finite_difference_of_runs": d, "fd_error": e, "adjoint_same_run": float(val),
                  "adjoint_error": err, "z": round((val - d) / float(np.hypot(e, err)), 2),
                  "adjoint_reweighted_32_runs": float(reweighted[k])}
    return out


def bench_plain_l16(steps, warmup, local, flush, cpu=True):
    """Plain small run: L=16, disordered start, T=0.815, P=0.45, 1 sweep + volume + cube per step.
    Launch-latency bound, so the per-step time inside a 32-step graph replay is reported too. With
    cpu, the oracle's steps/s on one host core over the first 2000 steps of the same chain, and
    whether its lattice after them equals the engine's."""
    import torch
    from cvfbulkwater_gb300.engine import Lattice, Params
    lat = Lattice(Params(L=16, T=0.815, P=0.45, seed=SEED, start=0, device=local))
    warm_steps(lat, warmup)
    ms = timed_steps(lat, steps, flush)
    stream = torch.cuda.ExternalStream(lat.stream_ptr())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        lat.run(32 * 20, 1, 0)
        e1.record(stream)
    torch.cuda.synchronize()
    replay_us = e0.elapsed_time(e1) * 1e3 / 640
    lat.close()
    # the small plain workload's protocol: 1000 equilibration + 10000 sampling steps, a record
    # every 10
    lat = Lattice(Params(L=16, T=0.815, P=0.45, seed=SEED, start=0, device=local))
    t0 = time.perf_counter()
    lat.run(1000, 1, 0)
    lat.run_sampled(10000, 1, 0, 10)
    smp = lat.samples()
    wall = time.perf_counter() - t0
    e, v, nhb = sample_columns(lat, smp)
    lat.close()

    def mean_err(x):
        b = x[: len(x) // 20 * 20].reshape(20, -1).mean(1)
        return [round(float(x.mean()), 6), round(float(b.std(ddof=1) / np.sqrt(20)), 6)]
    out = {"workload": "L=16 disordered start, T=0.815, P=0.45, 1 cube + 1 volume move + 1 sweep per step",
           "steps_per_s": round(steps / (ms / 1e3), 1), "site_updates_per_ns": round(4096 * steps / (ms * 1e6), 4),
           "graph_replay_us_per_step": round(replay_us, 3),
           "sampled_run": {"steps": 11000, "records": int(len(smp)), "wall_s": round(wall, 3),
                           "per_cell_mean_and_20_block_error": {
                               "E": mean_err(e / 4096), "V": mean_err(v / 4096), "rho": mean_err(4096 / v),
                               "N_hb": mean_err(nhb / 4096)}}}
    if cpu:
        from oracle import oracle as O
        n = 2000
        lat = Lattice(Params(L=16, T=0.815, P=0.45, seed=SEED, start=0, device=local))
        lat.run(n, 1, 0)
        o = O.Oracle(16, 0.815, 0.45, SEED, 6.0, 0, 0)
        t0 = time.perf_counter()
        for _ in range(n):
            o.step(1, 0)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"steps_per_s": round(n / dt, 1), "site_updates_per_ns": round(4096 * n / (dt * 1e9), 6),
                               "cores": 1, "kind": "port", "sample": f"the first {n} steps of the same chain",
                               "identical_lattice": bool(np.array_equal(lat.get_config(), o.get_config()))}
        lat.close()
        o.close()
    return out


def bench_sw(steps, warmup, local, flush):
    """Swendsen-Wang path: L=64 and L=128, T=0.60 and 0.75, P=0.45, disordered start,
    Cluster_Steps=1, Metropolis_Steps=0 (each step: cube move, volume move, one SW step)."""
    from cvfbulkwater_gb300.engine import Lattice, Params
    out = []
    for L in (64, 128):
        for T in (0.60, 0.75):
            lat = Lattice(Params(L=L, T=T, P=0.45, seed=SEED, start=0, device=local))
            warm_steps(lat, warmup, nmet=0, ncl=1)
            ms = timed_steps(lat, steps, flush, nmet=0, ncl=1)
            cs = lat.cluster_stats()
            out.append({"L": L, "T": T, "sw_steps_per_s": round(steps / (ms / 1e3), 1),
                        "site_updates_per_ns": round(L ** 3 * steps / (ms * 1e6), 4),
                        "labelling_passes_per_step": 1,
                        "algorithmic_GBps": round(68 * L ** 3 * steps / (ms / 1e3) / 1e9, 1),
                        "largest_cluster": int(cs.largest), "n_clusters": int(cs.n_clusters)})
            lat.close()
    return out


def bench_wolff(local):
    """Wolff cluster steps (GW:2199-2357, compiled out of the reference's default build): L=64 and
    L=128, T=0.60, P=0.45, disordered start, Cluster_Steps=1, Metropolis_Steps=0, against the
    oracle's sequential pokes on one host core (one step at L=64)."""
    import torch
    from cvfbulkwater_gb300.engine import Lattice, Params
    from oracle import oracle as O
    out = []
    for L, steps in ((64, 3), (128, 2)):
        lat = Lattice(Params(L=L, T=0.60, P=0.45, seed=SEED, start=0, device=local))
        lat.set_cluster_algorithm(True)
        lat.run(1, 0, 1)
        lat.synchronize()
        s = torch.cuda.ExternalStream(lat.stream_ptr(), device=f"cuda:{local}")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        lat.run(steps, 0, 1)
        e1.record(s)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        pokes, total, largest, _ = lat.wolff_stats()
        row = {"L": L, "T": 0.60, "ms_per_step": round(ms, 2), "pokes_per_step": pokes, "largest_cluster": largest,
               "pokes_per_us": round(pokes / (ms * 1e3), 2)}
        lat.close()
        if L == 64:
            o = O.Oracle(L, 0.60, 0.45, SEED, 6.0, 0, 0)
            o.set_wolff(True)
            o.step(0, 1)
            t0 = time.perf_counter()
            o.step(0, 1)
            row["cpu_baseline"] = {"ms_per_step": round((time.perf_counter() - t0) * 1e3, 1), "cores": 1,
                                   "kind": "port", "sample": "one Wolff step of the same L=64 lattice"}
        out.append(row)
    return out


def pinned_copy(a):
    """A copy of numpy array a in page-locked host memory (a numpy view of a pinned torch buffer)."""
    import torch
    t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
    out = t.numpy().view(a.dtype).reshape(a.shape)
    out[...] = a
    return out


def workload_config(n_gpus):
    """The `config` object both arms print: the same workload, so the lines compare one to one."""
    return {"workload": "L=256 ordered start, T=0.70, P=0.45, Metropolis only; 1 cube move + "
                        "1 volume move + 1 checkerboard sweep per step", "L": L_BENCH, "cells": L_BENCH ** 3,
            "l2": "64 MB lattice < 129 MB L2: a 256 MB buffer is written before every timed step",
            "replicas": n_gpus}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    cap = max(1, min(args.steps, 20))
    base = cpu_baseline_oracle(steps_cap=cap, budget_s=90.0)
    line = {"impl": "reference", "metric": "site-updates/ns at L=256", "value": base["value"],
            "unit": "site-updates/ns", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (ordered start, Philox seed 44648604 + rank)",
            "config": workload_config(args.gpus),
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": "site-updates/ns", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_engine(args):
    rank, world, local = dist_env()
    dist = Dist(world)
    import torch
    from cvfbulkwater_gb300 import build
    build.build()
    import ctypes as C
    from cvfbulkwater_gb300 import abi
    from cvfbulkwater_gb300.engine import Lattice, Params

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        base = cpu_baseline_oracle()

    torch.cuda.set_device(local)
    L = L_BENCH
    N = L ** 3
    lat = Lattice(replica_params(rank, local))
    stream = torch.cuda.ExternalStream(lat.stream_ptr(), device=local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    tile = lat.set_sweep_tile(args.tile) if args.tile else lat.autotune()
    warm_steps(lat, args.warmup)
    # roofline of the dominant kernel (the sweep), two launches per profiled sweep
    nprof = max(4, min(args.steps, 50))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nprof)]
    with torch.cuda.stream(stream):
        for i in range(nprof):
            flush.fill_(i & 255)
            ev[i][0].record(stream)
            abi.check(abi.lib().cvf_profile_launch(lat._h, 0, 1))
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    sweep_ms = sum(a.elapsed_time(b) for a, b in ev) / nprof
    launch_s = sweep_ms / 2 / 1e3
    alg_bytes_launch = ALG_BYTES_PER_CELL_SWEEP * N / 2

    # timed region: K steps, L2 flushed before each
    dist.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(i & 255)
            ev[i][0].record(stream)
            lat.run(1, 1, 0)
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    total_ms = dist.max(total_ms)
    ms_per_step = total_ms / args.steps
    value = world * N * args.steps / (total_ms * 1e6)

    # L2-resident reference figure: the same K steps back to back, no flush
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        lat.run(args.steps, 1, 0)
        e1.record(stream)
    torch.cuda.synchronize()
    resident = N * args.steps / (e0.elapsed_time(e1) * 1e6)

    # end to end through the C ABI with host buffers: upload a host configuration, then per step
    # one run call and one observables read (device -> host), finally download the lattice. The
    # headline uses the reference's own host arrays (s and active_bond, one byte per arm each:
    # what GW:1135-1137 copies to the device and GW:1298 copies back).
    lat2 = Lattice(Params(L=L, T=T_BENCH, P=P_BENCH, seed=SEED + 7 + rank, start=1, replica=rank, device=local))
    lat2.set_sweep_tile(tile)  # tuned once like the handle above (a fresh handle starts at 4 cells)
    # the caller's host buffers are page-locked (pinned) memory, filled before the timed region
    host_s, host_ab = (pinned_copy(x) for x in lat.get_arms())
    out_arms = (pinned_copy(np.zeros_like(host_s)), pinned_copy(np.zeros_like(host_ab)))  # reusable result buffers
    lat2.set_arms(host_s, host_ab)
    for _ in range(max(3, args.warmup)):
        lat2.run(1, 1, 0)
        lat2.observables()
    lat2.get_arms(out=out_arms)
    dist.barrier()
    t0 = time.perf_counter()
    lat2.set_arms(host_s, host_ab)
    ta = time.perf_counter()
    for _ in range(args.steps):
        lat2.run(1, 1, 0)
        lat2.observables()
    tb = time.perf_counter()
    lat2.get_arms(out=out_arms)
    t1 = time.perf_counter()
    arm_bytes = 12 * N  # s and active_bond, 6N bytes each
    e2e = {"value": round(world * N * args.steps / (dist.max(t1 - t0) * 1e9), 4), "unit": "site-updates/ns",
           "h2d_bytes_per_step": int(round(arm_bytes / args.steps)),
           "d2h_bytes_per_step": int(round(arm_bytes / args.steps)) + 32,
           "upload_ms": round(1e3 * (ta - t0), 3), "steps_ms": round(1e3 * (tb - ta), 3),
           "download_ms": round(1e3 * (t1 - tb), 3),
           "note": "per step: cvf_run_steps(1 step, measured on its colour-1 sweep) + cvf_observables (the record, 32 B D2H, sync); host buffers page-locked; "
                   "lattice upload (cvf_set_arms: the caller's s and active_bond arrays, 201 MB, read and "
                   "packed by the GPU in host memory) and download (cvf_get_arms: unpacked by the GPU into "
                   "the caller's arrays) amortised over the K steps"}
    # the same sequence through the config.out order (cells12: twelve int32 per cell)
    host_cfg = pinned_copy(lat.get_config())
    out_buf = pinned_copy(np.zeros_like(host_cfg))
    out_buf.fill(0)  # a caller's reusable result buffer
    # one untimed pass of the same sequence: the first GPU access to a host page (here the
    # result buffer's) sets up its translation, a one-time cost of a reused buffer
    lat2.set_config(host_cfg)
    for _ in range(max(3, args.warmup)):
        lat2.run(1, 1, 0)
        lat2.observables()
    lat2.get_config(out=out_buf)
    dist.barrier()
    t0 = time.perf_counter()
    lat2.set_config(host_cfg)
    ta = time.perf_counter()
    for _ in range(args.steps):
        lat2.run(1, 1, 0)
        lat2.observables()
    tb = time.perf_counter()
    out_cfg = lat2.get_config(out=out_buf)
    t1 = time.perf_counter()
    e2e_s = dist.max(t1 - t0)
    cells12_bytes = 12 * 4 * N  # what crosses the host link each way: the caller's int32 cells12 array
    e2e_cells12 = {"value": round(world * N * args.steps / (e2e_s * 1e9), 4), "unit": "site-updates/ns",
           "h2d_bytes_per_step": int(round(cells12_bytes / args.steps)),
           "d2h_bytes_per_step": int(round(cells12_bytes / args.steps)) + 32,
           "upload_ms": round(1e3 * (ta - t0), 3), "steps_ms": round(1e3 * (tb - ta), 3),
           "download_ms": round(1e3 * (t1 - tb), 3),
           "note": "per step: cvf_run_steps(1 step, measured on its colour-1 sweep) + cvf_observables (the record, 32 B D2H, sync); host buffers page-locked; "
                   "lattice upload (cvf_set_config: the caller's 805 MB cells12 array read and packed "
                   "by the GPU in host memory, io_mode 1) and download (cvf_get_config: unpacked by the "
                   "GPU into the caller's array) amortised over the K steps"}
    del out_cfg
    # the same sequence with the compact checkpoint format: cvf_set_packed + cvf_set_state in,
    # cvf_get_packed + cvf_get_state out (4.25 bytes per cell each way instead of 48)
    pk = pinned_copy(lat.get_packed())
    st = lat.state()
    pk_out = pinned_copy(np.zeros_like(pk))
    lat2.set_packed(pk)
    lat2.set_state(st[0], st[1], st[3])
    for _ in range(max(3, args.warmup)):
        lat2.run(1, 1, 0)
        lat2.observables()
    lat2.get_packed(out=pk_out)
    dist.barrier()
    t0 = time.perf_counter()
    lat2.set_packed(pk)
    lat2.set_state(st[0], st[1], st[3])
    ta = time.perf_counter()
    for _ in range(args.steps):
        lat2.run(1, 1, 0)
        lat2.observables()
    tb = time.perf_counter()
    lat2.get_packed(out=pk_out)
    lat2.state()
    t1 = time.perf_counter()
    e2e_packed = {"value": round(world * N * args.steps / (dist.max(t1 - t0) * 1e9), 4), "unit": "site-updates/ns",
                  "h2d_bytes_per_step": int(round((pk.size + 40) / args.steps)),
                  "d2h_bytes_per_step": int(round((pk.size + 40) / args.steps)) + 32,
                  "upload_ms": round(1e3 * (ta - t0), 3), "steps_ms": round(1e3 * (tb - ta), 3),
                  "download_ms": round(1e3 * (t1 - tb), 3),
                  "note": "as e2e with the packed checkpoint format: cvf_set_packed + cvf_set_state, per step "
                          "cvf_run_steps + cvf_observables, cvf_get_packed + cvf_get_state (71 MB each way)"}
    # the drop-in driver's production loop: one sampled run call recording a sample after every
    # step on the device, the K records read back afterwards (after an untimed short run of the
    # same calls)
    lat2.run_sampled(max(3, args.warmup), 1, 0, 1)
    lat2.samples()
    dist.barrier()
    t0 = time.perf_counter()
    lat2.set_arms(host_s, host_ab)
    lat2.clear_samples()
    ta = time.perf_counter()
    lat2.run_sampled(args.steps, 1, 0, 1)
    smp = lat2.samples()
    tb = time.perf_counter()
    lat2.get_arms(out=out_arms)
    t1 = time.perf_counter()
    e2e_sampled = {"value": round(world * N * args.steps / (dist.max(t1 - t0) * 1e9), 4),
                   "unit": "site-updates/ns", "records": int(len(smp)),
                   "upload_ms": round(1e3 * (ta - t0), 3), "steps_ms": round(1e3 * (tb - ta), 3),
                   "download_ms": round(1e3 * (t1 - tb), 3),
                   "note": "cvf_set_arms, cvf_run_sampled(K steps, a record after every step), "
                           "cvf_get_samples, cvf_get_arms"}

    extras = {"e2e_cells12": e2e_cells12, "e2e_sampled": e2e_sampled, "e2e_packed": e2e_packed}
    if rank == 0 and world == 1 and not args.no_extras:
        extras["batched"] = bench_batch64(max(10, min(args.steps, 50)), args.warmup, local, flush)
        extras["swendsen_wang"] = bench_sw(max(10, min(args.steps, 30)), args.warmup, local, flush)
        extras["wolff"] = bench_wolff(local)
        extras["plain_l16"] = bench_plain_l16(max(10, min(args.steps, 50)), args.warmup, local, flush,
                                              cpu=not args.no_cpu_baseline)
        extras["differentiation"] = bench_differentiation(local)
        if not args.no_cpu_baseline:
            extras["cpu_baseline_1thread"] = cpu_baseline_oracle(steps_cap=1, budget_s=10.0, threads=1)

    peak, peak_kind = peaks()
    achieved = alg_bytes_launch / launch_s / 1e9
    traffic = ncu_traffic("sweep_l256_traffic.json", tile)
    sm_mhz = (clk or {}).get("sm_mhz") or 2070.0
    issue = issue_roof(tile, N // 2, launch_s, sm_mhz, torch.cuda.get_device_properties(local).multi_processor_count)
    line = {
        "metric": "site-updates/ns at L=256", "value": round(value, 4), "unit": "site-updates/ns",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
        "data": "synthetic (ordered start, Philox seed 44648604 + rank)",
        "config": workload_config(world),
        "sweep_tile": tile,
        "tuning": dict(zip(("tile", "lg_rows", "launch_mode"), lat.tuning())),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "kernel": f"k_sweep<{tile}> (one colour of the checkerboard sweep)",
                     "algorithmic_bytes_per_launch": int(alg_bytes_launch),
                     "launch_us": round(launch_s * 1e6, 3), "peak_source": f"{peak_kind} hbm_gbs",
                     "issue": issue},
        "cpu_baseline": base,
        "e2e": e2e,
        "gpu_launches": 4 * args.steps,
        "clocks": clk,
        "l2_resident_value": round(resident, 4),
        "arm_updates_per_ns": round(6 * value, 4),
    }
    line.update(extras)
    if rank == 0:
        print(json.dumps(line), flush=True)
    lat.close()
    lat2.close()
    dist.close()
    return 0

def _timed(fn, reps=1):
    """Wall seconds of the fastest of reps calls of fn (which synchronizes itself)."""
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return best


def run_analysis(args):
    """One JSON line for the analysis stages built around the step loop: the isobar run
    statistics, the multi-tau correlator and the 2-D reweighting search, each on the GPU through
    the library and as the oracle's CPU restatement (one host thread, a bounded sample, scaled
    to the same unit)."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    import torch
    from cvfbulkwater_gb300 import build as b
    b.build()
    from cvfbulkwater_gb300.analysis import Histogram2D, f90_range
    from cvfbulkwater_gb300.engine import Lattice, Params
    from oracle import correlator as OC
    from oracle import hist2d as OH
    from oracle import isobar as OI
    torch.cuda.set_device(local)
    rows = {}

    # isobar run statistics: 64 replicas of L=16 (the isobar sizes' smallest), 20,000 records each
    R, L, K = 64, 16, 20000
    lat = Lattice([Params(L=L, T=0.6 + 0.005 * i, P=0.45, seed=700 + i, start=0, replica=i, device=local)
                   for i in range(R)])
    lat.run(200, 1, 0)
    lat.run_sampled(K, 1, 0, 1)
    lat.synchronize()
    t_gpu = _timed(lambda: lat.run_statistics(), reps=5)
    cols = []
    for s in lat.samples(0)[:4000]:
        o = lat.sample_observables(s, 0)
        cols.append([o.energy, o.enthalpy, o.v_total, o.n_hb, o.m, o.r_cell])
    cols = np.array(cols)
    t_cpu = _timed(lambda: OI.run_stats(cols))
    lat.close()
    rows["isobar_run_statistics"] = {
        "workload": f"mean and variance of the six data.out columns over {K} records of each of {R} replicas "
                    f"(L={L}), read from the on-device sample stream",
        "gpu": {"value": round(R * K / t_gpu / 1e6, 3), "unit": "M records/s"},
        "cpu_baseline": {"value": round(len(cols) / t_cpu / 1e6, 4), "unit": "M records/s", "cores": 1,
                         "kind": "port", "sample": f"{len(cols)} records of one replica (the awk sums in file order)"}}

    # multi-tau correlator on the bench lattice: per-step cost of the sigma histogram + correlator
    lat = Lattice(Params(L=L_BENCH, T=T_BENCH, P=P_BENCH, seed=SEED, start=2, device=local))
    lat.run(20, 1, 0)
    lat.synchronize()
    n = 200
    t_off = _timed(lambda: (lat.run(n, 1, 0), lat.synchronize()), reps=3)
    lat.set_correlation(True)
    t_on = _timed(lambda: (lat.run(n, 1, 0), lat.synchronize()), reps=3)
    lat.set_correlation(False)
    cells = lat.get_config()
    lat.close()
    mt = OC.MultiTau()
    nc = 5

    def cpu_corr():
        for _ in range(nc):
            mt.add(OC.max_mass(cells))
    t_cpu = _timed(cpu_corr)
    rows["multi_tau_correlator"] = {
        "workload": f"per MC step: histogram of the 6N sigma arms of the L={L_BENCH} lattice and one correlator "
                    "update (Flag_correlation = 1)",
        "gpu": {"value": round(max(t_on - t_off, 0.0) / n * 1e6, 2), "unit": "us/step",
                "note": "extra time of run(200) with the correlator on, device-resident lattice"},
        "cpu_baseline": {"value": round(t_cpu / nc * 1e6, 1), "unit": "us/step", "cores": 1, "kind": "port",
                         "sample": f"{nc} steps on a host copy of the lattice (the reference copies it to the host "
                                   "every step; that copy is not counted)"}}

    # 2-D histogram reweighting search of the F90 on 8 engine chains (L=8, T = 0.70 .. 0.77,
    # P = 0.45), 50,000 records each, bin_factor 1
    That = np.array([float(np.float32(0.70 + 0.01 * j)) for j in range(8)])
    ns = 50000
    lat = Lattice([Params(L=8, T=float(t), P=0.45, seed=900 + j, start=0, replica=j, device=local)
                   for j, t in enumerate(That)])
    lat.run(2000, 1, 0)
    lat.run_sampled(ns, 1, 0, 1)
    h, rho, run = [], [], []
    for j in range(8):
        for smp in lat.samples(j):
            ob = lat.sample_observables(smp, j)
            h.append(ob.enthalpy / 512.0)
            rho.append(512.0 / ob.v_total)
            run.append(j)
    lat.close()
    h, rho, run = np.array(h), np.array(rho), np.array(run)
    That = That.copy()
    Phat = np.full(8, float(np.float32(0.45)))
    o = OH.H2D(h, rho, run, That, Phat, 8, 1.0)
    n_it = 1500
    t0 = time.perf_counter()
    H = Histogram2D(h, rho, run, That, Phat, 8, bin_factor=1.0, steps=n_it, device=local)
    t_wham = time.perf_counter() - t0
    o.ctes = H.ctes.copy()  # the oracle reweights with the converged constants

    def cpu_wham_step():
        try:
            o.wham(1)
        except RuntimeError:  # one step from zero has not converged; only its time counts
            pass
    t_wham_cpu = _timed(cpu_wham_step)
    o.ctes = H.ctes.copy()
    T = f90_range(0.72, 0.76, 0.01)
    P = np.array([0.45])
    S = f90_range(-0.5, 0.5, 0.05, inclusive=False)
    t_gpu = _timed(lambda: H.scan(T, P, S), reps=2)
    t_cpu = _timed(lambda: OH.scan(o, T[:1], P, S[:4]))
    nbm = H.n_bin_mixed
    H.close()
    n_gpu, n_cpu = len(T) * len(P) * len(S), 4
    rows["hist2d_search"] = {
        "workload": f"F90 search over {len(T)} T x {len(P)} P x {len(S)} angles: reweighted {o.nb}x{o.nb} grid "
                    f"(8 engine chains, L=8, x {ns} records, bin_factor 1), mixed parameter ({nbm} bins), Binder cumulants "
                    "and Ising comparisons per angle",
        "gpu": {"value": round(n_gpu / t_gpu, 1), "unit": "(T, P, angle) rows/s"},
        "cpu_baseline": {"value": round(n_cpu / t_cpu, 2), "unit": "(T, P, angle) rows/s", "cores": 1,
                         "kind": "port", "sample": "1 (T, P) point x 4 angles (one reweighting + 4 mixed histograms)"},
        "constants": {"gpu": {"value": round(n_it / t_wham, 1), "unit": "iterations/s",
                              "note": f"{n_it} iterations of the 8 runs' constants incl. binning the samples"},
                      "cpu_baseline": {"value": round(1 / t_wham_cpu, 3), "unit": "iterations/s", "cores": 1,
                                       "kind": "port", "sample": "1 iteration"}}}
    line = {"metric": "analysis stages around the step loop (isobar statistics, correlator, 2-D reweighting)",
            "impl": "engine", "n_gpus": 1, "data": "synthetic", "rows": rows}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and Swendsen-Wang sub-benchmarks")
    ap.add_argument("--tile", type=int, default=0,
                    help="sweep tile (cells per thread) instead of the autotuner's choice, e.g. to profile one tile")
    ap.add_argument("--analysis", action="store_true",
                    help="print one line timing the analysis stages (GPU against the oracle) instead")
    args = ap.parse_args()
    if args.analysis:
        return run_analysis(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_engine(args)


if __name__ == "__main__":
    sys.exit(main())
