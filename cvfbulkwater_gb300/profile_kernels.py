"""Launches one kernel kind of the engine a fixed number of times, for profilers.

  python -m cvfbulkwater_gb300.profile_kernels --L 256 --kind sweep --launches 2

Creates one lattice (ordered start, T=0.70, P=0.45), runs --warmup full Monte Carlo steps
and then --launches profiled repetitions of the chosen kind: a single kernel kind through
cvf_profile_launch (sweep = 2 launches per repetition), or whole steps (kind "step": cube +
volume + sweep; kind "step_sw": cube + volume + one Swendsen-Wang step; --correlation adds
the multi-tau correlator's histogram and update to every step).
Prints the mean time per repetition measured with CUDA events on the engine's stream.
"""
from __future__ import annotations

import argparse
import ctypes as C

KINDS = {"sweep": 0, "cube": 1, "volume": 2, "measure": 3}
STEPS = {"step": (1, 0), "step_sw": (0, 1)}  # full MC steps: (Metropolis sweeps, SW steps)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--L", type=int, default=256)
    ap.add_argument("--kind", default="sweep", choices=sorted(KINDS) + sorted(STEPS))
    ap.add_argument("--launches", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--start", type=int, default=2)
    ap.add_argument("--T", type=float, default=0.70)
    ap.add_argument("--P", type=float, default=0.45)
    ap.add_argument("--mode", type=int, default=None, help="launch mode of the step kinds (0 per phase, 1 persistent)")
    ap.add_argument("--correlation", action="store_true",
                    help="step kinds with the multi-tau correlator on (Flag_correlation = 1)")
    a = ap.parse_args()
    import torch

    from . import abi, build
    from .engine import Lattice, Params
    build.build()
    lat = Lattice(Params(L=a.L, T=a.T, P=a.P, seed=44648604, start=a.start))
    if a.mode is not None:
        lat.launch_mode = a.mode
    if a.correlation:
        lat.set_correlation(True)
    nmet, ncl = STEPS.get(a.kind, (1, 0))
    lat.run(a.warmup, nmet, ncl)
    lat.synchronize()
    sp = C.c_void_p()
    abi.check(abi.lib().cvf_get_stream(lat._h, C.byref(sp)))
    s = torch.cuda.ExternalStream(sp.value)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    if a.kind in STEPS:
        lat.run(a.launches, nmet, ncl)
    else:
        abi.check(abi.lib().cvf_profile_launch(lat._h, KINDS[a.kind], a.launches))
    e1.record(s)
    torch.cuda.synchronize()
    print(f"L={a.L} kind={a.kind} mode={lat.launch_mode} repetitions={a.launches} "
          f"ms/rep={e0.elapsed_time(e1) / max(a.launches, 1):.4f}")
    lat.synchronize()
    lat.close()


if __name__ == "__main__":
    main()
