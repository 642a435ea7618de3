"""Launches one kernel kind of the engine a fixed number of times, for profilers.

  python -m cvfbulkwater_gb300.profile_kernels --L 256 --kind sweep --launches 2

Creates one lattice (ordered start, T=0.70, P=0.45), runs --warmup full Monte Carlo steps
and then --launches profiled repetitions of the chosen kind: a single kernel kind through
cvf_profile_launch (sweep = 2 launches per repetition), or whole steps (kind "step": cube +
volume + sweep; kind "step_sw": cube + volume + one Swendsen-Wang step; kind "step_wolff": cube +
volume + one Wolff step; --correlation adds
the multi-tau correlator's histogram and update to every step). Kind "batch64" runs the steps of
the 64-replica batch (L drawn from {16,24,32,48,64} with seed 20261203, the 8x8 grid T 0.55..0.95
x P 0..0.60, disordered starts, seeds 44648604 + replica) with the 4-cell sweep tile.
Prints the mean time per repetition measured with CUDA events on the engine's stream. Kind
"c2c" times the configuration transfers against plain copies over the host link, kind
"h2d_scan" the 2-D reweighting search.
"""
from __future__ import annotations

import argparse
import ctypes as C

KINDS = {"sweep": 0, "cube": 1, "volume": 2, "measure": 3}
ANALYSIS = ("h2d_scan", "c2c")
# full MC steps: (Metropolis sweeps, cluster steps); step_wolff's cluster steps are Wolff steps
STEPS = {"step": (1, 0), "step_sw": (0, 1), "step_wolff": (0, 1), "batch64": (1, 0)}


def batch64_params():
    """The 64-replica batch: L drawn from {16,24,32,48,64}, T on 8 points of [0.55, 0.95], P on 8
    points of [0, 0.60], disordered starts."""
    import numpy as np

    from .engine import Params
    rng = np.random.default_rng(20261203)
    Ls = rng.choice([16, 24, 32, 48, 64], size=64)
    Ts = np.linspace(0.55, 0.95, 8)
    Ps = np.linspace(0.0, 0.60, 8)
    return [Params(L=int(Ls[i]), T=float(Ts[i % 8]), P=float(Ps[i // 8]), seed=44648604 + i, start=0, replica=i)
            for i in range(64)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--L", type=int, default=256)
    ap.add_argument("--kind", default="sweep", choices=sorted(KINDS) + sorted(STEPS) + list(ANALYSIS))
    ap.add_argument("--launches", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--start", type=int, default=2)
    ap.add_argument("--T", type=float, default=0.70)
    ap.add_argument("--P", type=float, default=0.45)
    ap.add_argument("--mode", type=int, default=None, help="launch mode of the step kinds (0 per phase, 1 persistent)")
    ap.add_argument("--nhb", action="store_true",
                    help="step kinds in the nhb<=4 compatibility mode (Flag_chessboard = 0)")
    ap.add_argument("--measure", action="store_true",
                    help="step kinds followed by one observables read per repetition")
    ap.add_argument("--correlation", action="store_true",
                    help="step kinds with the multi-tau correlator on (Flag_correlation = 1)")
    a = ap.parse_args()
    import torch

    from . import abi, build
    from .engine import Lattice, Params
    build.build()
    if a.kind == "h2d_scan":
        return h2d_scan(a)
    if a.kind == "c2c":
        return c2c(a)
    if a.kind == "batch64":
        lat = Lattice(batch64_params())
        lat.set_sweep_tile(4)
    else:
        lat = Lattice(Params(L=a.L, T=a.T, P=a.P, seed=44648604, start=a.start, flag_chessboard=0 if a.nhb else 1))
    if a.mode is not None:
        lat.launch_mode = a.mode
    if a.correlation:
        lat.set_correlation(True)
    if a.kind == "step_wolff":
        lat.set_cluster_algorithm(True)
    nmet, ncl = STEPS.get(a.kind, (1, 0))
    lat.run(a.warmup, nmet, ncl)
    lat.synchronize()
    sp = C.c_void_p()
    abi.check(abi.lib().cvf_get_stream(lat._h, C.byref(sp)))
    s = torch.cuda.ExternalStream(sp.value)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    if a.kind in STEPS and a.measure:
        for _ in range(a.launches):
            lat.run(1, nmet, ncl)
            lat.observables()
    elif a.kind in STEPS:
        lat.run(a.launches, nmet, ncl)
    else:
        abi.check(abi.lib().cvf_profile_launch(lat._h, KINDS[a.kind], a.launches))
    e1.record(s)
    torch.cuda.synchronize()
    print(f"L={a.L} kind={a.kind} mode={lat.launch_mode} repetitions={a.launches} "
          f"ms/rep={e0.elapsed_time(e1) / max(a.launches, 1):.4f}")
    lat.synchronize()
    lat.close()


def h2d_scan(a):
    """The 2-D reweighting search on 8 chains of L=--L lattices at T = 0.70 .. 0.77 (20,000 records
    each, bin_factor 1, 1500 constant iterations), then --launches searches over 5 temperatures x
    21 angles."""
    import time

    import numpy as np

    from .analysis import Histogram2D, f90_range
    from .engine import Lattice, Params
    That = np.array([float(np.float32(0.70 + 0.01 * j)) for j in range(8)])
    lat = Lattice([Params(L=a.L, T=float(t), P=a.P, seed=900 + j, start=0, replica=j) for j, t in enumerate(That)])
    lat.run(2000, 1, 0)
    lat.run_sampled(20000, 1, 0, 1)
    N = float(a.L) ** 3
    h, rho, run = [], [], []
    for j in range(8):
        for smp in lat.samples(j):
            ob = lat.sample_observables(smp, j)
            h.append(ob.enthalpy / N)
            rho.append(N / ob.v_total)
            run.append(j)
    lat.close()
    H = Histogram2D(np.array(h), np.array(rho), np.array(run), That, np.full(8, float(np.float32(a.P))), a.L,
                    bin_factor=1.0, steps=1500)
    T, P, S = f90_range(0.72, 0.76, 0.01), np.array([a.P]), f90_range(-0.5, 0.5, 0.05, inclusive=False)
    t0 = time.perf_counter()
    for _ in range(max(a.launches, 1)):
        H.scan(T, P, S)
    dt = (time.perf_counter() - t0) / max(a.launches, 1)
    print(f"h2d_scan L={a.L} grid={H.n_bin2d}^2 rows={len(T) * len(S)} ms/search={dt * 1e3:.2f}")
    H.close()


def c2c(a):
    """The host link under the configuration transfers: a plain copy of an (L^3, 12) int32 array in
    pageable host memory to and from the device (cudaMemcpy through torch), against
    cvf_set_config / cvf_get_config of the same array (the GPU packing and unpacking it in place),
    each the best of --launches repetitions after one untimed pass."""
    import time

    import numpy as np
    import torch

    from .engine import Lattice, Params
    lat = Lattice(Params(L=a.L, T=a.T, P=a.P, seed=44648604, start=1))
    cfg = lat.get_config()
    buf = np.empty_like(cfg)
    buf.fill(0)
    nbytes = cfg.nbytes
    host = torch.from_numpy(buf.reshape(-1))
    dev = torch.empty(host.numel(), dtype=torch.int32, device="cuda")

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(max(a.launches, 1)):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best

    h2d = timed(lambda: dev.copy_(host))
    d2h = timed(lambda: host.copy_(dev))
    up = timed(lambda: lat.set_config(cfg))
    down = timed(lambda: lat.get_config(out=buf))
    for name, t in (("copy H2D", h2d), ("copy D2H", d2h), ("cvf_set_config", up), ("cvf_get_config", down)):
        print(f"c2c L={a.L} {name}: {t * 1e3:.3f} ms, {nbytes / t / 1e9:.1f} GB/s of the {nbytes / 1e6:.0f} MB array")
    lat.close()


if __name__ == "__main__":
    main()
