"""Command line: advance a named Yin-Yang MHD workload on a GPU and print the
device time per step.

    python -m falcon_gb300 --workload shell_fp64_442k --steps 10 --warmup 3
    python -m falcon_gb300 --workload shell_mixed_21m --steps 20

Workloads:
  shell_fp64_442k  plain FP64 shell, per panel 32 x 48 x 144 cells in 8^3
                   blocks (864 blocks, 442,368 cells), bit-identical to the oracle
  shell_fp64_21m   the 21,233,664-cell shell (16^3 blocks) in FP64
  shell_mixed_21m  the same shell in the mixed precision of the benchmark
  shell_mixed_5m   the same physics at 1/4 of the blocks (1,296 blocks of 16^3,
                   5,308,416 cells): the profiling case
Initial state: kind 1 of falcon_init_synthetic (entropy bump, dipole B and a
random-phase Kolmogorov velocity at rms Mach 0.01, seed 1002).

--tuning KS KD fixes the k-chunk variants of the stage and diffusion kernels
(falcon_set_tuning) instead of the autotuner, whose timings a profiler would
distort; --step-mode persistent runs each step as one persistent launch.
--end-to-end times, per step, the core of the FP64 state uploaded from pinned,
page-aligned host memory (falcon_upload_state_core), the step, and the core
downloaded again (falcon_download_state_core): the median of each part.
"""
import argparse
import json
import sys

import time

from . import Falcon, build, config, host_array

WORKLOADS = {
    "shell_fp64_442k": lambda d: config.shell_fp64_cpu(device=d),
    "shell_fp64_21m": lambda d: config.shell_mixed_21m(precision=config.PREC_FP64, device=d),
    "shell_mixed_21m": lambda d: config.shell_mixed_21m(device=d),
    "shell_mixed_5m": lambda d: config.make_config(block=(16, 16, 16), root_tiles=(3, 3, 9), radial_levels=1,
                                                   radial_option=1, amr=((0, 1, 1),), precision=config.PREC_MIXED,
                                                   device=d),
}


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m falcon_gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="shell_fp64_442k")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--tuning", type=int, nargs=2, metavar=("KS", "KD"), default=None)
    ap.add_argument("--step-mode", choices=("graph", "persistent"), default="graph")
    ap.add_argument("--end-to-end", action="store_true")
    a = ap.parse_args(argv)
    build()
    f = Falcon(WORKLOADS[a.workload](a.device))
    if a.tuning:
        f.set_tuning(*a.tuning)
    if a.step_mode == "persistent":
        from . import STEP_PERSISTENT
        f.set_step_mode(STEP_PERSISTENT)
    f.init_synthetic(kind=1, seed=1002, mach=0.01)
    if a.end_to_end:
        return end_to_end(f, a)
    f.exchange()
    f.exchange()
    f.run_steps(a.warmup)
    f.synchronize()
    f.timer_start()
    f.run_steps(a.steps)
    ms = f.timer_stop()
    f.synchronize()
    print(json.dumps({"workload": a.workload, "cells": f.interior_cells, "steps": a.steps, "step_mode": a.step_mode,
                      "ms_per_step": ms / max(a.steps, 1),
                      "cell_updates_per_s": f.interior_cells * a.steps / (ms / 1e3) if ms > 0 else None,
                      "tuning": f.tuning()}))
    f.close()
    return 0


def end_to_end(f, a):
    import numpy as np
    host = host_array(f.shape)
    f.pin_host(host)
    f.download_state_into(host)
    f.synchronize()
    parts = {"upload": [], "step": [], "download": []}
    for s in range(a.warmup + a.steps):
        t0 = time.perf_counter()
        f.upload_state_core(host)
        t1 = time.perf_counter()
        f.advance_rk4(want_dt=True)
        f.synchronize()
        t2 = time.perf_counter()
        f.download_state_core(host)
        t3 = time.perf_counter()
        if s >= a.warmup:
            for k, t in (("upload", t1 - t0), ("step", t2 - t1), ("download", t3 - t2)):
                parts[k].append(t)
    f.unpin_host(host)
    med = {k: float(np.median(v)) * 1e3 for k, v in parts.items()}
    tot = sum(med.values())
    core = host[:, :, 2:-2, 2:-2, :].nbytes
    print(json.dumps({"workload": a.workload, "cells": f.interior_cells, "steps": a.steps, "end_to_end_ms": med,
                      "core_bytes": core, "upload_gb_s": core / med["upload"] / 1e6,
                      "download_gb_s": core / med["download"] / 1e6, "ms_per_step": tot,
                      "cell_updates_per_s": f.interior_cells / (tot / 1e3) if tot > 0 else None,
                      "tuning": f.tuning()}))
    f.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
