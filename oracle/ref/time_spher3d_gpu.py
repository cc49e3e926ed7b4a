"""Times the reference's own sfAWEFDspher3Dgpu (built unchanged for sm_103a by
oracle/ref/Makefile.gpu) beside the drop-in sfAWEFDspher3Dgpu on the
spherical-shell configuration: r 700 x theta 512 x phi 512 (764 x 576 x 576
padded), nb 32, one Ricker source at 50 m altitude and 64 x 64 receivers,
expl=n, free=n (the reference's free-surface kernel writes past the end of
its last line), traces every step.  Each program runs twice, with nt1 and
nt2 steps; the difference of the wall times over nt2 - nt1 is the time per
step, so reading the inputs and setting up cancel.  The traces of the two
programs at nt2 are compared (rel-L2), for the engine's AWE_FAST and
AWE_EXACT arithmetic (the reference evaluates cos/sin of theta on the GPU per
cell, the engine from host tables).

Test infrastructure, run on a GPU machine after the build:

    make -C oracle/ref -f Makefile.gpu && python oracle/ref/time_spher3d_gpu.py [nt1 nt2]

Prints one JSON line.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from wavefield_imaging_gb300 import build as awe_build  # noqa: E402
from wavefield_imaging_gb300 import rsf  # noqa: E402

REF_BIN = os.path.join(ROOT, "oracle", "_ref", "sfAWEFDspher3Dgpu_ref")


def write_inputs(tmp, nt):
    w = bench.spher_workload(nt)
    vel = bench.spher_model(w)
    sou, rec = bench.spher_shots(w, 1)[0]
    rsf.write(os.path.join(tmp, "vel.rsf"), vel, [(n, o, d) for n, o, d in zip(w["n"], w["o"], w["d"])])
    rsf.write(os.path.join(tmp, "sou.rsf"), sou, [(3, 0.0, 1.0), (1, 0.0, 1.0)])
    rsf.write(os.path.join(tmp, "rec.rsf"), rec, [(3, 0.0, 1.0), (rec.shape[0], 0.0, 1.0)])
    return w, rec.shape[0]


def run(binary, tmp, nt, w, label, precision="fast"):
    t = np.arange(nt) * w["dt"] - 0.1
    a = (np.pi * w["f0"] * t) ** 2
    wav = ((1 - 2 * a) * np.exp(-a)).astype(np.float32).reshape(nt, 1)
    wpath = os.path.join(tmp, "wav_%d.rsf" % nt)
    rsf.write(wpath, wav, [(1, 0.0, 1.0), (nt, 0.0, w["dt"])])
    out = os.path.join(tmp, "dat_%s_%d.rsf" % (label, nt))
    args = [binary, "vel=" + os.path.join(tmp, "vel.rsf"), "sou=" + os.path.join(tmp, "sou.rsf"),
            "rec=" + os.path.join(tmp, "rec.rsf"), "nb=%d" % w["nb"], "expl=n", "free=n", "snap=n", "jdata=1",
            "gpu=0", "wfl=" + os.path.join(tmp, "wfl_%s.rsf" % label)]
    if label != "reference":
        args.append("precision=" + precision)
    with open(wpath, "rb") as fin, open(out, "wb") as fout:
        t0 = time.perf_counter()
        r = subprocess.run(args, stdin=fin, stdout=fout, stderr=subprocess.PIPE, timeout=1200)
        secs = time.perf_counter() - t0
    if r.returncode != 0:
        raise RuntimeError("%s failed: %s" % (label, r.stderr.decode()[-2000:]))
    dat, _ = rsf.read(out)
    return secs, dat


def main():
    nt1, nt2 = (int(sys.argv[1]), int(sys.argv[2])) if len(sys.argv) > 2 else (20, 220)
    eng_bin = os.path.join(awe_build.build_programs(), "sfAWEFDspher3Dgpu")
    with tempfile.TemporaryDirectory() as tmp:
        w, nr = write_inputs(tmp, nt2)
        res = {}
        for label, binary in (("reference", REF_BIN), ("engine", eng_bin)):
            s1, _ = run(binary, tmp, nt1, w, label)
            s2, d2 = run(binary, tmp, nt2, w, label)
            res[label] = dict(s_nt1=s1, s_nt2=s2, ms_per_step=1e3 * (s2 - s1) / (nt2 - nt1), traces=d2)
        _, exact = run(eng_bin, tmp, nt2, w, "engine_exact", precision="exact")
    cells = int(np.prod([n + 2 * w["nb"] for n in w["n"]]))
    ref = res["reference"]["traces"].astype(np.float64).ravel()

    def rel_to_ref(x):
        x = np.asarray(x, np.float64).ravel()
        n = min(ref.size, x.size)
        return float(np.linalg.norm(x[:n] - ref[:n]) / max(np.linalg.norm(ref[:n]), 1e-300)), n

    rel, n = rel_to_ref(res["engine"]["traces"])
    rel_exact, _ = rel_to_ref(exact)
    out = {"workload": "spherical shell 700 x 512 x 512 (764 x 576 x 576 padded), nb 32, 1 source, %d receivers, "
                       "expl=n free=n, traces every step" % nr,
           "nt": [nt1, nt2], "padded_cells": cells,
           "reference_gpu_program": {"ms_per_step": res["reference"]["ms_per_step"],
                                     "cell_updates_per_s": cells / (res["reference"]["ms_per_step"] / 1e3),
                                     "wall_s": [res["reference"]["s_nt1"], res["reference"]["s_nt2"]],
                                     "build": "CODE/MAWEFDspher3Dgpu.cu unchanged, nvcc -prec-div=true "
                                              "-arch=sm_103a --x=cu"},
           "engine_program": {"ms_per_step": res["engine"]["ms_per_step"],
                              "cell_updates_per_s": cells / (res["engine"]["ms_per_step"] / 1e3),
                              "wall_s": [res["engine"]["s_nt1"], res["engine"]["s_nt2"]]},
           "speedup": res["reference"]["ms_per_step"] / res["engine"]["ms_per_step"],
           "traces_rel_l2_engine_vs_reference_gpu": rel,
           "traces_rel_l2_engine_exact_vs_reference_gpu": rel_exact, "trace_samples_compared": n}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
