"""Autotuner of the tall tensor-core kernels' schedule and tile parameters.

The parameters (plom_set_tuning, include/plom.h) are the Gram's work items
per SM per wave (row-chunk granularity; narrow and wide Grams each their
own), the resident blocks per SM of the
Gram's slab reduction, the output tile width of dense products wider than
128 columns, whether those products give each CTA whole row blocks and the
row chunks of a large FP32 input packed beside the first Gram and the
products that run on SM pairs.
On the GPU at hand the tuner times the mixed-form tsqr_svd with CUDA events
on two snapshot fields of the POD benchmark's kind -- a wide one (2 x rows
points, n = 1,024: the 128 x 256 Gram and apply kernels) and a narrow one
(rows points, n = 64: the 128 x 128 kernels) -- and settles one parameter at a time (coordinate
descent from the current values, two passes), keeping a value only when it
is faster on the sum of the two shapes' median times relative to the
starting point.  The result is written as JSON, which the package applies
at load (pyloworder_gb300/tuning/gb300.json unless PLOM_TUNING names
another file):

    python -m pyloworder_gb300.autotune [--out PATH] [--rows M] [--reps R]
"""
from __future__ import annotations

import argparse
import json
import os
import time

CANDIDATES = {
    "gram_wave_mult": [1, 2, 4, 8],
    "gram_wide_wave_mult": [8, 16, 32, 64, 128],
    "reduce_blocks_per_sm": [2, 3, 4],
    "apply_dense_tn": [128, 256],
    "apply_dense_by_rows": [0, 1],
    "apply_tri_by_rows": [0, 1],
    "pass1_chunks": [1, 4, 8],
    "apply_pair": [0, 1, 2],
}


def _fields(rows):
    from . import datagen, vmmath
    out = []
    for n, m in ((1024, 2 * rows), (64, rows)):
        rows_n = m
        nx, ny = datagen.grid_for_points(rows_n)
        X = datagen.pod_field_device(nx, ny, n, min(64, n // 2), seed=17 + n, noise=1e-5,
                                     amp_pow=1.5, m=rows_n)
        Y, _, _ = vmmath.remove_mean_device(X, n)
        del X
        out.append((f"tsqr_svd {rows_n}x{n} f32 mixed", Y, n))
    return out


def _time(lib, fields, reps):
    """Median ms per call of each field's tsqr_svd (after one untimed call)."""
    import torch

    from . import vmmath
    times = []
    for _, Y, n in fields:
        vmmath.tsqr_svd_device(Y, n, "mixed")
        ms = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            vmmath.tsqr_svd_device(Y, n, "mixed")
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        times.append(sorted(ms)[len(ms) // 2])
    return times


def tune(rows=2_097_152, reps=5, passes=2, log=print):
    import torch

    from . import _lib as L
    lib = L.load()
    fields = _fields(rows)
    current = {k: int(lib.plom_get_tuning(k.encode())) for k in CANDIDATES}
    base = _time(lib, fields, reps)
    log(f"start {current}: {base}")

    def score(t):
        return sum(a / b for a, b in zip(t, base))

    best = score(base)
    trials = []
    for _ in range(passes):
        for key, values in CANDIDATES.items():
            for v in values:
                if v == current[key]:
                    continue
                L.call("plom_set_tuning", key.encode(), float(v))
                t = _time(lib, fields, reps)
                sc = score(t)
                trials.append({"params": {**current, key: v}, "ms": t, "score": sc})
                log(f"{key}={v}: {t} score {sc:.4f} (best {best:.4f})")
                if sc < best * 0.995:
                    best, current[key] = sc, v
                L.call("plom_set_tuning", key.encode(), float(current[key]))
    final = _time(lib, fields, reps)
    return {
        "device": torch.cuda.get_device_name(0),
        "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
        "params": current,
        "workloads": [f[0] for f in fields],
        "start_ms": base,
        "final_ms": final,
        "trials": trials,
        "method": "coordinate descent over CANDIDATES from the library defaults, "
                  f"{passes} passes, median of {reps} calls per shape, a change kept "
                  "when the sum of the shapes' time ratios drops by more than 0.5 %",
    }


def main():
    from . import _lib as L
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=L.TUNING_FILE)
    ap.add_argument("--rows", type=int, default=2_097_152)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--passes", type=int, default=2)
    args = ap.parse_args()
    os.environ["PLOM_TUNING"] = ""  # start from the library's defaults
    res = tune(args.rows, args.reps, args.passes)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    with open(args.out, "w") as f:
        json.dump(res, f, indent=1)
    print(json.dumps({"params": res["params"], "start_ms": res["start_ms"],
                      "final_ms": res["final_ms"]}))


if __name__ == "__main__":
    main()
