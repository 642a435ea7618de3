"""Regenerates the golden fixtures of tests/golden/ from the reference checkout.

Run in a container where the reference repository lcoronas/CVFBulkWater is mounted (its path is
the first argument). The fixtures are outputs and inputs that ship with the reference, reduced
to what the tests need:

  distances_L32_Rc6.txt     SOURCE/distances (vdW shell table written by gpu_water3D, L=32, Rc=6)
  input_config_L32.npz      SOURCE/input_config (32768 cells x 12 ints) as uint8
  config_out_L32.npz        SOURCE/config.out, same format
  input_data.txt            SOURCE/input_data (the 14-line parameter file)
  water3D.log               SOURCE/water3D.log (log format)
  cluster_out_head.txt      first 5 lines of SOURCE/cluster.out (format; Cluster_Steps = 0)
  data_out_head.txt         first 5 lines of SOURCE/data.out (format)
  data_out_stats.json       means and 20-block errors of data.out columns 2-7 (L=32, T=0.815,
                            P=0.45, 10000 samples): the statistical golden of the engine
  isobar_P0.45_density.txt  PROCESSED_DATA/CVF_isobars.tar.gz: L32_P0.45_density.dat
  isobars_L32.txt           every isobar of the same archive, one line per point:
                            P T rho err (L32_P*_density.dat, calculadora.sh output)
  isobars_L32_si.txt        P T_K rho_SI err_SI (L32_P*_density.dat.SI, conversor.sh:20)
  isobars_L32_alphap_si.txt P T_K alpha_P err (L32_P*_AlphaPderivate.dat.SI, conversor.sh:54-66
                            with AlphaPderivate.c), the printed text kept as it is
  isobars_L32_kt_si.txt     P_MPa T_K K_T err P_MPa (L32_P*_KTderivate.dat.SI, conversor.sh:84-119
                            with KTderivate.c, isobars named by their pressure in MPa), as printed
  correlator_ref.json       the reference's own multi-tau correlator (initialize/add/evaluate of
                            SOURCE/gpu_water3D.cu, built by oracle/build_ref.py) on a seeded
                            random walk of 20000 values: the evaluated (t, f), as hex floats
"""
from __future__ import annotations

import io
import json
import os
import sys
import tarfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def blocking(x, nb=20):
    x = np.asarray(x, dtype=np.float64)
    b = x[: len(x) // nb * nb].reshape(nb, -1).mean(1)
    return float(x.mean()), float(b.std(ddof=1) / np.sqrt(nb)), float(x.std())


def main(ref: str):
    src = os.path.join(ref, "SOURCE")
    with open(os.path.join(src, "distances")) as f:
        open(os.path.join(HERE, "distances_L32_Rc6.txt"), "w").write(f.read())
    for name, out in [("input_config", "input_config_L32.npz"), ("config.out", "config_out_L32.npz")]:
        a = np.loadtxt(os.path.join(src, name), dtype=np.int64).astype(np.uint8)
        np.savez_compressed(os.path.join(HERE, out), cells12=a)
    for name, out in [("input_data", "input_data.txt"), ("water3D.log", "water3D.log")]:
        open(os.path.join(HERE, out), "w").write(open(os.path.join(src, name)).read())
    for name, out in [("cluster.out", "cluster_out_head.txt"), ("data.out", "data_out_head.txt")]:
        with open(os.path.join(src, name)) as f:
            lines = [next(f) for _ in range(5)]
        open(os.path.join(HERE, out), "w").write("".join(lines))
    d = np.loadtxt(os.path.join(src, "data.out"))
    stats = {"source": "SOURCE/data.out", "L": 32, "T": 0.815, "P": 0.45, "rows": int(len(d)),
             "interval": 10, "columns": {}}
    for col, name in [(1, "e"), (2, "h"), (3, "v"), (4, "n_hb"), (5, "m"), (6, "r_cell")]:
        m, err, sd = blocking(d[:, col])
        stats["columns"][name] = {"mean": m, "block_err": err, "std": sd}
    json.dump(stats, open(os.path.join(HERE, "data_out_stats.json"), "w"), indent=1)
    with tarfile.open(os.path.join(ref, "PROCESSED_DATA", "CVF_isobars.tar.gz")) as t:
        m = t.getmember("CVF_isobars/L32_P0.45_density.dat")
        data = t.extractfile(m).read().decode()
    open(os.path.join(HERE, "isobar_P0.45_density.txt"), "w").write(data)
    kinds = [("density.dat", "isobars_L32.txt"), ("density.dat.SI", "isobars_L32_si.txt"),
             ("AlphaPderivate.dat.SI", "isobars_L32_alphap_si.txt"), ("KTderivate.dat.SI", "isobars_L32_kt_si.txt")]
    with tarfile.open(os.path.join(ref, "PROCESSED_DATA", "CVF_isobars.tar.gz")) as t:
        names = t.getnames()
        for suffix, out in kinds:
            lines = []
            for n in sorted(names):
                base = os.path.basename(n)
                if not (base.startswith("L32_P") and base.endswith("_" + suffix)):
                    continue
                P = base[len("L32_P"):-len("_" + suffix)]
                for line in t.extractfile(n).read().decode().splitlines():
                    if line.strip():
                        lines.append(P + " " + line.strip())
            open(os.path.join(HERE, out), "w").write("\n".join(lines) + "\n")
    correlator_golden(ref)


def correlator_input():
    rng = np.random.default_rng(20261203)
    return 0.5 + 0.01 * np.cumsum(rng.standard_normal(20000))


def correlator_golden(ref):
    import ctypes as C
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle import build_ref
    lib = build_ref.build(ref)
    if lib is None:
        return
    L = C.CDLL(lib)
    w = np.ascontiguousarray(correlator_input())
    t, f = np.zeros(512), np.zeros(512)
    n = L.ref_corr_run(w.ctypes.data_as(C.c_void_p), len(w), t.ctypes.data_as(C.c_void_p),
                       f.ctypes.data_as(C.c_void_p), 512)
    json.dump({"source": "SOURCE/gpu_water3D.cu initialize/add/evaluate (GW:2983-3107), norm=1",
               "input": "0.5 + 0.01*cumsum(numpy default_rng(20261203).standard_normal(20000))",
               "t": [float(x).hex() for x in t[:n]], "f": [float(x).hex() for x in f[:n]]},
              open(os.path.join(HERE, "correlator_ref.json"), "w"), indent=0)


if __name__ == "__main__":
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle import build_ref

    ref = build_ref.checkout(sys.argv[1] if len(sys.argv) > 1 else None)
    if ref is None:
        sys.exit("no reference checkout: pass its path or set CVF_REFERENCE_DIR")
    main(ref)
