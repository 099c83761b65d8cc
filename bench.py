"""Benchmark: MHD cell-updates/s per RK4 step on the 21M-cell mixed-precision shell.

Workload: Yin-Yang spherical shell r in [0.7, 1.0] R_sun, per panel 96 x 192 x 576
cells in 16^3 blocks (5,184 blocks, 21,233,664 cells), 8 variables, polytrope
background (n = 1.5, density contrast 100), seeded entropy bump + dipole B +
random-phase Kolmogorov velocity (rms Mach 0.01). One "step" is one full
ModAdvance_rk4: CFL reduction, four RK stages with a ghost exchange after each,
the artificial-diffusion pass and its exchange. FP32 state and stencil RHS,
FP64 p1 assembly, CFL reduction and dt.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N>1 (under torchrun): every rank advances its own replica of the shell on its
GPU ("replicas only": the shell is not partitioned across GPUs); value is the
sum of cell-updates over ranks divided by the max time over ranks.

--impl reference times the CPU restatement of the reference algorithm (the
oracle's -O3 timing build; the Fortran reference cannot be built here) on the
host cores, on the same 21,233,664-cell workload (a few steps, median), plus a
1-core run on a 442,368-cell shell, and prints the same JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "MHD cell-updates/s per RK4 step"
UNIT = "cell-updates/s"
STATE_BYTES_PER_VAR = 4          # FP32 stored state
CORR_BYTES_PER_VAR = 1           # 8-bit correction of u^n
NVAR = 8
# algorithmic bytes per interior cell per RK4 step (the workload's stated
# figure B = nvar*s*14 + 6*s): 4 stages x (read u_s, read u^n, write u_s+1) +
# diffusion (read, write) = 14 state passes of 8 variables, plus the CFL read
# of v and B. The mixed path's u^n correction (read and written by stage 4
# and the diffusion pass, 32 B) is traffic of this design, not of the figure.
BYTES_PER_CELL_STEP = NVAR * STATE_BYTES_PER_VAR * 14 + 6 * STATE_BYTES_PER_VAR   # 472
CORR_BYTES_PER_CELL_STEP = NVAR * CORR_BYTES_PER_VAR * 4                          # 32
# per launch, on the same basis
STAGE_BYTES_PER_CELL = NVAR * STATE_BYTES_PER_VAR * 3   # 96
DIFF_BYTES_PER_CELL = NVAR * STATE_BYTES_PER_VAR * 2    # 64
WORKLOAD = "yinyang_shell_mhd_21M_mixed"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(name):
    """DRAM bytes per launch from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch_full_size:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []   # (arrival time, line)
        self.window = None

    def start(self):
        """Start sampling (every 50 ms) and wait for the first sample, so that
        the window marked by begin()/end() is covered from its start."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.perf_counter()
            while not self.lines and time.perf_counter() - t0 < 10.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def begin(self):
        self.window = [time.perf_counter(), None]

    def end(self):
        if self.window:
            self.window[1] = time.perf_counter()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.06)   # the sample that closes the window
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        rows = self.lines
        if self.window and self.window[1] is not None:
            a, b = self.window
            inside = [r for r in rows if a <= r[0] <= b]
            after = [r for r in rows if r[0] > b][:1]   # a sample taken at the window's end
            rows = inside + after if inside or after else rows
        for _, ln in rows:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    """torchrun env -> (rank, world, local_rank, dist module or None)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        return rank, world, local, dist
    return 0, 1, 0, None


def barrier(dist):
    if dist is not None:
        dist.barrier()


def reduce_max(dist, x):
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, x):
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def cpu_sample_config():
    """The 1-core CPU sample: the same physics in 16^3 blocks, per panel
    32 x 48 x 144 cells (108 blocks, 442,368 cells)."""
    from falcon_gb300 import config
    return config.make_config(block=(16, 16, 16), root_tiles=(1, 3, 9), radial_levels=1, radial_option=1,
                              amr=(), precision=config.PREC_FP64, device=-1)


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def _time_oracle_steps(cfg, max_steps, budget_s, threads=None):
    """Median seconds per step of the oracle's -O3 timing build on cfg (one
    warm-up step first), with `threads` OpenMP threads (None: all)."""
    import oracle
    from falcon_gb300 import synth
    oracle.build()
    if threads is not None:
        oracle.set_threads(threads, timing=True)
    try:
        o = oracle.Oracle(cfg, timing=True)
        u0 = synth.initial_state(cfg, o.block_ranges(), o.block_flags(), seed=1002)
        o.set_state(u0)
        del u0
        o.exchange()
        o.exchange()
        o.step()
        times, t_all = [], time.perf_counter()
        while len(times) < max_steps:
            t0 = time.perf_counter()
            o.step()
            times.append(time.perf_counter() - t0)
            if time.perf_counter() - t_all > budget_s:
                break
        cores = oracle.num_threads(timing=True)
        cells = o.nblocks * cfg.tree.ni * cfg.tree.nj * cfg.tree.nk
        del o
        return statistics.median(times), len(times), cores, cells
    finally:
        if threads is not None:
            oracle.set_threads(os.cpu_count() or 1, timing=True)


def time_cpu_reference(max_steps=5, budget_s=60.0):
    """The CPU restatement of the reference step (the oracle; the Fortran
    reference cannot be built here), timing build (-O3, OpenMP over blocks),
    on the machine's host cores: the full 21,233,664-cell workload with every
    thread, median of up to `max_steps` steps after one warm-up step; and on
    one core, the 442,368-cell sample shell, median of 5 steps."""
    from falcon_gb300 import config
    full = config.shell_mixed_21m(precision=config.PREC_FP64, device=-1)
    med, n, cores, cells = _time_oracle_steps(full, max_steps, budget_s)
    med1, n1, _, cells1 = _time_oracle_steps(cpu_sample_config(), 5, 30.0, threads=1)
    return {"value": cells / med, "unit": UNIT, "cores": cores, "kind": "port",
            "build": "oracle -O3 timing build (oracle/build/liboracle_fast.so), OpenMP over blocks",
            "sample": "full workload: %d cells (5,184 blocks of 16^3), median of %d steps after 1 warm-up step; "
                      "initial state: entropy bump + dipole B (the step's cost does not depend on the values)"
                      % (cells, n),
            "s_per_step": med,
            "cores_1": {"value": cells1 / med1, "unit": UNIT, "cores": 1, "s_per_step": med1,
                        "sample": "%d-cell shell (108 blocks of 16^3), median of %d steps" % (cells1, n1)},
            "cpu_model": cpu_model(), "nproc": os.cpu_count()}


def run_reference(args, rank, world, dist):
    if rank != 0:
        return
    cpu = time_cpu_reference(max_steps=max(min(args.steps, 5), 3))
    value = cpu["value"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": 21233664, "blocks": 5184, "block": [16, 16, 16],
                   "same_config": True, "timed": cpu["sample"]},
        "impl": "reference",
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def small_config(device):
    """Profiling case: the same shell and physics at 1/4 of the blocks per
    panel (per panel 96 x 96 x 288 cells, 1,296 blocks of 16^3, 332 MB per
    FP32 state buffer: larger than L2 but a few GB on the device)."""
    from falcon_gb300 import config
    return config.make_config(block=(16, 16, 16), root_tiles=(3, 3, 9), radial_levels=1, radial_option=1,
                              amr=((0, 1, 1),), precision=config.PREC_MIXED, device=device)


def run_ours(args, rank, world, local, dist):
    import falcon_gb300 as fg
    from falcon_gb300 import config
    fg.build()
    cfg = config.shell_mixed_21m(device=local) if args.workload == "full" else small_config(local)
    t_setup = time.perf_counter()
    f = fg.Falcon(cfg)   # tree, block geometry, ghost map (host), device tables and lists
    setup_s = time.perf_counter() - t_setup
    cells = f.interior_cells
    f.init_synthetic(kind=1, seed=1002, mach=0.01)
    f.exchange()
    f.exchange()
    # ---- device-resident throughput (value)
    f.run_steps(args.warmup)
    f.synchronize()
    barrier(dist)
    f.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    f.synchronize()
    clocks.begin()
    f.timer_start()
    f.run_steps(args.steps)
    ms = f.timer_stop()
    f.synchronize()
    clocks.end()
    clk = clocks.stop()
    barrier(dist)
    ms_max = reduce_max(dist, ms)
    total_cells = reduce_sum(dist, float(cells * args.steps))
    value = total_cells / (ms_max / 1e3)
    lists = f.ghost_list_sizes()

    # ---- per-kernel times (events around every launch) for the roofline
    f.set_kernel_timing(True)
    f.reset_kernel_stats()
    f.run_steps(2)
    f.synchronize()
    stats = f.kernel_stats()
    f.set_kernel_timing(False)
    # launches per step, counted by the context's per-kernel timing over those
    # 2 steps: finalize_dt (the CFL minimum comes from the previous step's
    # diffusion pass), 4 stages and the diffusion pass, and after each of
    # them the exchange of the ghost entries the kernels do not push
    launches_per_step = int(round(sum(v[1] for v in stats.values()) / 2.0))
    tot = sum(v[0] for v in stats.values()) or 1.0
    top = max(stats, key=lambda k: stats[k][0])
    avg_ms = stats[top][0] / max(stats[top][1], 1)
    ghosts = sum(lists.values())
    per_cell = {"stage": STAGE_BYTES_PER_CELL, "diffusion": DIFF_BYTES_PER_CELL}.get(top)
    if top == "ghost_fill":
        # one exchange: every ghost cell reads and writes its 8 variables (FP32)
        per_cell = ghosts * NVAR * 2 * STATE_BYTES_PER_VAR / cells
    hbm, peak_kind = peaks()
    roof = None
    if per_cell is not None:
        ach = cells * per_cell / (avg_ms / 1e3) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                "traffic": profile_traffic("%s_mixed_21m.txt" % top), "kernel": top,
                "algorithmic_bytes_per_launch": cells * per_cell, "avg_launch_ms": avg_ms,
                "peak_kind": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind}
    # ---- the same step as one persistent cooperative launch (the kernel
    # bodies over all blocks with grid barriers between the phases); timed
    # like the graph above, on the same context
    try:
        f.set_step_mode(fg.STEP_PERSISTENT)
        f.run_steps(args.warmup)
        f.synchronize()
        f.timer_start()
        f.run_steps(args.steps)
        pms = reduce_max(dist, f.timer_stop())
        f.synchronize()
        f.set_step_mode(fg.STEP_GRAPH)
        persistent = {"ms_per_step": pms / args.steps, "launches_per_step": 1,
                      "value": reduce_sum(dist, float(cells * args.steps)) / (pms / 1e3)}
    except fg.FalconError as ex:
        f.set_step_mode(fg.STEP_GRAPH)
        persistent = {"unavailable": str(ex)}
    step_modes = {"graph": {"ms_per_step": ms_max / args.steps, "launches_per_step": launches_per_step},
                  "persistent": persistent}
    step_ach = cells * BYTES_PER_CELL_STEP / (ms_max / args.steps / 1e3) / 1e9
    shares = {k: round(v[0] / tot, 4) for k, v in stats.items()}

    # ---- end to end through the C ABI with host buffers: every step uploads
    # the FP64 Fortran-layout state from pinned host memory, advances, and
    # downloads the new state (the drop-in keeps Tree%LocalBlocks authoritative).
    # Headline: core transfers (interior planes x interior rows of every block
    # and variable; theta/phi ghost layers recomputed on the device); also the
    # whole padded array moved both ways.
    e2e_val = res_val = full_val = None
    nbytes = full_bytes = 0
    k_e2e = max(1, min(args.steps, 10))
    if not args.no_e2e:
        host = fg.host_array(f.shape)   # 4096-byte aligned: whole 64-byte lines over the host link
        f.pin_host(host)
        f.download_state_into(host)
        f.synchronize()

        def e2e_loop(up, down):
            barrier(dist)
            t0 = time.perf_counter()
            for _ in range(k_e2e):
                up(host)
                f.advance_rk4(want_dt=True)
                down(host)
            dt_s = reduce_max(dist, time.perf_counter() - t0)
            return reduce_sum(dist, float(cells * k_e2e)) / dt_s

        e2e_val = e2e_loop(f.upload_state_core, f.download_state_core)
        full_val = e2e_loop(f.upload_state_raw, f.download_state_into)
        f.unpin_host(host)
        full_bytes = host.nbytes
        nbytes = host[:, :, 2:-2, 2:-2, :].size * 8
        # resident variant: the state stays on the GPU, dt comes back every step
        t0 = time.perf_counter()
        for _ in range(k_e2e):
            f.advance_rk4(want_dt=True)
        res_s = reduce_max(dist, time.perf_counter() - t0)
        res_val = reduce_sum(dist, float(cells * k_e2e)) / res_s

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline and args.workload == "full":
        cpu = time_cpu_reference(max_steps=5, budget_s=40.0)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "cells": cells, "blocks": f.nblocks, "block": [16, 16, 16],
                       "ghost_layers": 2, "nvar": 8, "precision": "mixed",
                       "l2": "inputs larger than L2 (state %.0f MB per buffer)" % (cells * 8 * 4 * (20 / 16) ** 3 / 1e6),
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": roof,
            "step_roofline": {"achieved": step_ach, "peak": hbm, "unit": "GB/s", "frac": step_ach / hbm,
                              "algorithmic_bytes_per_cell_step": BYTES_PER_CELL_STEP,
                              "not_counted": "u^n correction, %d B/cell-step" % CORR_BYTES_PER_CELL_STEP},
            "kernel_time_share": shares,
            "tuning": f.tuning(), "ghost_lists": lists, "stage_exchange": f.exchange_stats(),
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                    "mode": "core of the FP64 state (interior planes x interior rows, pinned, 4096-byte aligned) "
                            "uploaded and downloaded every step; theta/phi ghost layers recomputed on the device"},
            "e2e_full_array": {"value": full_val, "unit": UNIT, "h2d_bytes_per_step": full_bytes,
                               "d2h_bytes_per_step": full_bytes,
                               "mode": "whole padded FP64 state (pinned) uploaded and downloaded every step"},
            "setup_s": round(setup_s, 3),
            "e2e_resident": {"value": res_val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 8},
            "gpu_launches": launches_per_step * args.steps,
            "step_modes": step_modes,
            "clocks": clk,
        }
    f.close()
    if rank == 0:
        if world == 1 and not args.no_accuracy and args.workload == "full":
            line["accuracy"] = accuracy_leg(local, steps=100)
            line["fp64_path"] = fp64_path_bench(local, line["accuracy"])
        if world == 1 and not args.no_solvers and args.workload == "full":
            line["solvers"] = solver_bench(local)
        print(json.dumps(line))


def accuracy_leg(device, steps=100):
    """The workload's accuracy: the same 21,233,664-cell shell and seeded
    initial state advanced `steps` RK4 steps in MIXED and in FP64 on the GPU
    (each with its own dt), per-variable relative L2 and norm-wise max error
    of the mixed state against the FP64 state over the interior cells
    (falcon_gb300.compare). The FP64 run is timed too (CUDA events)."""
    import falcon_gb300 as fg
    from falcon_gb300 import config
    from falcon_gb300.compare import state_errors, worst
    states, ms = {}, {}
    for name, prec in (("fp64", config.PREC_FP64), ("mixed", config.PREC_MIXED)):
        f = fg.Falcon(config.shell_mixed_21m(precision=prec, device=device))
        f.init_synthetic(kind=1, seed=1002, mach=0.01)
        f.exchange()
        f.exchange()
        f.advance_rk4(want_dt=False)    # first step: autotuner and graph capture
        f.synchronize()
        f.init_synthetic(kind=1, seed=1002, mach=0.01)
        f.exchange()
        f.exchange()
        f.synchronize()
        f.timer_start()
        f.run_steps(steps)
        ms[name] = f.timer_stop()
        f.synchronize()
        states[name] = f.download_state()
        cells = f.interior_cells
        f.close()
    e = state_errors(states["mixed"], states["fp64"])
    del states
    return {"workload": WORKLOAD, "cells": cells, "steps": steps, "seed": 1002, "init": "kind 1 (Kolmogorov, Mach 0.01)",
            "reference": "FP64 GPU path, same initial state", "per_var": e,
            "max_rel_l2": worst(e, "rel_l2"), "max_rel_max": worst(e, "rel_max"), "target_rel": 1e-6,
            "ms_per_step": {k: v / steps for k, v in ms.items()}}


def fp64_path_bench(device, acc):
    """Throughput of the FP64 (bit-exact) path: the 21M-cell shell from the
    accuracy run, and the 442,368-cell shell of 8^3 blocks (the CPU-runnable
    workload, 10 steps after 3 warm-up steps)."""
    import falcon_gb300 as fg
    from falcon_gb300 import config
    out = {}
    ms = acc["ms_per_step"]["fp64"]
    out["shell_21M_16cube"] = {"cells": acc["cells"], "ms_per_step": ms, "value": acc["cells"] / (ms / 1e3),
                               "bytes_per_cell_step": 944,
                               "achieved_GBs": acc["cells"] * 944 / (ms / 1e3) / 1e9}
    f = fg.Falcon(config.shell_fp64_cpu(device=device))
    f.init_synthetic(kind=0, seed=1001)
    f.exchange()
    f.exchange()
    f.run_steps(3)
    f.synchronize()
    f.timer_start()
    f.run_steps(10)
    t = f.timer_stop() / 10
    out["shell_442k_8cube"] = {"cells": f.interior_cells, "ms_per_step": t, "value": f.interior_cells / (t / 1e3),
                               "bytes_per_cell_step": 944,
                               "achieved_GBs": f.interior_cells * 944 / (t / 1e3) / 1e9}
    f.close()
    out["unit"] = UNIT
    return out


def _smooth_field(shape, rs):
    x = rs.normal(size=shape)
    for ax in (1, 2, 3):
        for _ in range(3):
            x = (x + np.roll(x, 1, axis=ax) + np.roll(x, -1, axis=ax)) / 3.0
    return x


def lcc_kernel_bench(x, t, device, reps=20):
    """The learned correction's network on one training batch (8 panels of
    16x32x96 coarse cells) through the host API, per tensor-core path: a
    forward pass and a loss-and-gradient pass (wall time per call, inputs
    copied in and results out), and one training step (device-resident)."""
    from falcon_gb300 import lcc as L
    out = {}
    for path, name in ((L.TCGEN05, "tcgen05"), (L.MMA_SYNC, "mma_sync")):
        net = L.LCC(device=device, seed=3)
        net.set_tensor_path(path)
        net.forward(x)
        net.loss_grad(x, t)
        t0 = time.perf_counter()
        for _ in range(reps):
            net.forward(x)
        fwd = (time.perf_counter() - t0) / reps
        t0 = time.perf_counter()
        for _ in range(reps):
            net.loss_grad(x, t)
        bwd = (time.perf_counter() - t0) / reps
        X, T = np.repeat(x, 4, axis=0), np.repeat(t, 4, axis=0)
        net.train(X, T, epochs=1, batch=8, lr=1e-4, seed=1)
        t0 = time.perf_counter()
        net.train(X, T, epochs=5, batch=8, lr=1e-4, seed=1)
        step = (time.perf_counter() - t0) / 20
        out[name] = {"forward_ms": round(fwd * 1e3, 3), "loss_grad_ms": round(bwd * 1e3, 3),
                     "train_step_ms": round(step * 1e3, 3)}
        net.close()
    return out


def solver_bench(device):
    """The implicit-solver workloads, each solved once after a warm-up solve:
    conduction MG-PCG at 64x128x384 cells per panel, the learned coarse
    correction against MG-PCG at 96x192x576 (trained on records of 64x128x384
    solves with other seeds and right-hand sides), and the batch of 64 PFSS
    problems. Times are CUDA-event times of the solve on the device."""
    from falcon_gb300 import solver as S
    from falcon_gb300.lcc import LCC
    out = {}
    t0 = time.time()
    sv = S.Solver(S.conduction_spec(seed=3001, device=device))
    sv.solve(tol=1e-8, max_iter=300, precond=S.PRECOND_MG, check=False)
    mg = sv.solve(tol=1e-8, max_iter=300, precond=S.PRECOND_MG, check=False)
    cg = sv.solve(tol=1e-8, max_iter=3000, precond=S.PRECOND_NONE, check=False)
    out["conduction_64x128x384"] = {"cells": sv.nblocks * sv.nint, "tol": 1e-8, "mg_pcg": mg, "plain_cg": cg,
                                     "tile": sv.tuning()}
    sv.close()
    # 2,000 training pairs (one panel's coarsest-level residual and exact
    # coarse error each) from real solves of the 64x128x384 system: systems
    # seeded 2000, 2001, ... (T and B), 8 smooth right-hand sides each
    X, T, npairs, s = [], [], 2000, 0
    t_rec = time.time()
    while sum(len(x) for x in X) < npairs:
        sv = S.Solver(S.conduction_spec(seed=2000 + s, device=device))
        rs = np.random.default_rng(200 + s)
        for r in range(8):
            sv.set_rhs(sv.apply(_smooth_field((sv.nblocks,) + sv.m[::-1], rs)))
            x, t = sv.record(tol=1e-8, max_iter=100, max_records=16)
            X.append(x)
            T.append(t)
            if sum(len(x) for x in X) >= npairs:
                break
        sv.close()
        s += 1
    X, T = np.concatenate(X)[:npairs], np.concatenate(T)[:npairs]
    record_s = time.time() - t_rec
    net = LCC(device=device, seed=11)
    t1 = time.time()
    losses = net.train(X, T, epochs=20, batch=8, lr=1e-3, seed=3)
    train_s = time.time() - t1
    lcc_kernels = lcc_kernel_bench(X[:8], T[:8], device)
    sv = S.Solver(S.conduction_spec(nr=96, nt=192, np_=576, seed=9999, device=device))
    sv.attach_lcc(net, sweeps=2)
    res = {}
    for pc, name in ((S.PRECOND_MG, "mg_pcg"), (S.PRECOND_MG_LCC, "learned_fcg")):
        sv.solve(tol=1e-8, max_iter=600, precond=pc, check=False)
        res[name] = sv.solve(tol=1e-8, max_iter=600, precond=pc, check=False)
    out["learned_vs_mg_96x192x576"] = {
        "cells": sv.nblocks * sv.nint, "tol": 1e-8, "training_pairs": int(len(X)), "training_systems": s,
        "record_s": round(record_s, 2), "train_s": round(train_s, 2), "train_epochs": 20,
        "tensor_path": "tcgen05", "network_kernels": lcc_kernels,
        "epoch_loss_first_last": [float(losses[0]), float(losses[-1])], **res,
        "time_ratio_learned_over_mg": res["learned_fcg"]["ms"] / res["mg_pcg"]["ms"]}
    sv.close()
    sizes = S.random_pfss_sizes(64, seed=5000)
    sv = S.Solver(S.pfss_spec(sizes, device=device))
    rep = sv.solve(tol=1e-10, max_iter=300, precond=S.PRECOND_MG, check=False)
    rel = sv.problem_residuals()
    out["pfss_batch64"] = {"problems": 64, "cells": sv.nblocks * sv.nint, "tol": 1e-10, "mg_pcg": rep,
                           "fp64_residual_per_problem": {"max": float(rel.max()), "median": float(np.median(rel))},
                           "tile": sv.tuning(),
                           "graph_launches": "one per inner solve (a device-side WHILE loop of FCG iterations, "
                                             "V-cycle included), one FP64 residual check per refinement pass"}
    sv.close()
    out["wall_s"] = round(time.time() - t0, 1)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the 100-step mixed-vs-FP64 accuracy run reported under 'accuracy'")
    ap.add_argument("--no-solvers", action="store_true",
                    help="skip the implicit-solver workloads reported under 'solvers'")
    ap.add_argument("--workload", default="full", choices=["full", "small"],
                    help="small: the 1,296-block profiling case (not a bench line)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    rank, world, local, dist = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world, dist)
    else:
        run_ours(args, rank, world, local, dist)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
