#!/usr/bin/env python
"""Benchmark: STS DOF-stages/s and time-to-solution at 8192^2, mixed vs FP64 GPU.

Workload (the configuration the headline metric is quoted on): the manufactured 2-D heat
problem u_t = kx u_xx + ky u_yy + b on [0,1]^2, 8192 x 8192 interior nodes (67.1M DOF),
kx = 1, ky = 1e-2, RKL2 super-time-stepping with adaptive steps (rtol 1e-6, atol 1e-10,
at most 200 stages), t in [0, 0.05]; inputs are synthetic (the analytic initial state).

A "step" is one adaptive LSRK time step (s fused stencil+stage kernels, the fused step-end
kernel and the host step control). value = DOF-stages/s of the mixed path (FP32 stage
increments, FP64 step update) with the state resident in HBM; e2e = the same metric through
the C-ABI with the state copied in from pinned host memory and back out every step;
"fp64" gives the plain FP64 GPU path replaying the mixed arm's step sequence, so both end at
the same t and "accuracy" compares their fields. Each FP32 stage buffer is
256 MiB (> 129 MB L2), so no L2 flush is needed between steps.

--impl reference times the CPU restatement of the reference algorithm (the oracle, FP64,
all host threads) on the same workload: the same adaptive RKL2 run from t = 0, the same
warm-up and timed step counts.
--full runs the whole t in [0, 0.05] solve for both precisions (time-to-solution).
"""
import argparse
import ctypes as C
import json
import math
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 8192
TF = 0.05
KX, KY = 1.0, 1e-2
RTOL, ATOL = 1e-6, 1e-10
METHOD = 1  # RKL2
SMAX = 200


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampler for the timed region (clocks and throttle reasons)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def merge_clocks(parts):
    """Clock record over the timed regions (mixed, FP64 and end to end)."""
    sm = [p["sm_mhz"] for p in parts if p.get("sm_mhz") is not None]
    mx = [p["sm_max_mhz"] for p in parts if p.get("sm_max_mhz") is not None]
    reasons = sorted(set(r for p in parts for r in p.get("reasons", [])))
    return {"sm_mhz": sorted(sm)[len(sm) // 2] if sm else None, "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons, "samples": sum(p.get("samples", 0) for p in parts),
            "per_region_sm_mhz": sm}


def cuda_timer(stream_ptr):
    import torch
    s = torch.cuda.ExternalStream(stream_ptr)

    class T:
        def __enter__(self):
            self.e0 = torch.cuda.Event(enable_timing=True)
            self.e1 = torch.cuda.Event(enable_timing=True)
            self.e0.record(s)
            return self

        def __exit__(self, *a):
            self.e1.record(s)
            self.e1.synchronize()
            self.ms = self.e0.elapsed_time(self.e1)
    return T


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of the mixed stage
# kernel, from one ncu capture of a smaller case of the same kernel, scaled to 8192^2 by the
# DOF count (the kernel streams each input once, so its traffic grows with the DOF count):
#   python bench.py --n 6144 --steps 1 --warmup 3 --no-cpu --stage-kernel 6
#   ncu --set full --clock-control none -k regex:stage32_tma -s 20 -c 2 -o prof_tma \
#       python bench.py --n 6144 --steps 1 --warmup 3 --no-cpu --stage-kernel 6
# 6144^2: 578.6 MB per launch -> x (8192/6144)^2 = 1028.7 MB.
TRAFFIC_MIXED_STAGE_6144 = 578.6e6


def mixed_stage_traffic(n):
    return TRAFFIC_MIXED_STAGE_6144 * (n / 6144.0) ** 2


# DRAM bytes of one launch of the fused four-stage kernel (120 x 64 tiles, two CTAs per SM,
# with d_{j-2} input), same method: a 6144^2 capture scaled by the DOF count:
#   python bench.py --n 6144 --steps 1 --warmup 3 --no-cpu --stage-fusion 4 --fusion-config 2
#   ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,dram__bytes_write.sum \
#       --clock-control none -k regex:stage32_fused -s 10 -c 2 --csv --log-file ncu_fused_6144.csv \
#       python bench.py --n 6144 --steps 1 --warmup 3 --no-cpu --stage-fusion 4 --fusion-config 2
# 6144^2: 459.5 MB read + 260.0 MB written = 719.5 MB per launch (algorithmic 754.9 MB).
TRAFFIC_FUSED4_6144 = 719.5e6


def fused_stage_traffic(n):
    return TRAFFIC_FUSED4_6144 * (n / 6144.0) ** 2


def step_launches(stages, ks):
    """Kernels one step attempt of `stages` stages launches on the fused mixed path: stage 1,
    the stages 2..s one per launch (ks = 1) or in groups of ks with a shorter last group (a
    last group of one stage runs as a single-stage launch), and the step end."""
    if ks <= 1:
        return stages + 1
    return 2 + (stages - 2 + ks) // ks


def replica_barrier(ws):
    """Host barrier of the N-replica run (one process per GPU, gloo): no data-path collective."""
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def replica_max(x, ws):
    """The slowest rank's time: every rank's timed region is bracketed by the barrier."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_gpu(args):
    import numpy as np
    import ceda_demonstrations_gb300 as sts

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    import torch
    torch.cuda.set_device(local)
    ctx = sts.Context(local)
    timer = cuda_timer(ctx.stream)
    n = args.n
    G = sts.Problem(ctx, sts.MANUFACTURED, n, n, KX, KY)
    N2 = n * n

    def barrier():
        replica_barrier(ws)

    def max_over_ranks(x):
        return replica_max(x, ws)

    res = {}
    clock_samples = []
    hseq = []  # accepted step sizes of the mixed arm, replayed by the FP64 arm
    L = sts.lib()
    for mixed in (True, False):
        I = sts.LSRKStep(ctx, G, 0.0, G.initial(), method=METHOD, rtol=RTOL, atol=ATOL,
                         smax=SMAX, mixed=mixed, graphs=True, maxsteps=1000000,
                         stage_kernel=args.stage_kernel if mixed else 0,
                         stage_fusion=(args.stage_fusion, args.fusion_config) if mixed else (1, 0))
        y = G.vector()

        step_stages = []  # stages_total after each mixed step: the stage count of every attempt

        def one_step(k):
            # the FP64 arm takes the mixed arm's step sequence (ARKodeSetFixedStep before each
            # step), so that both end at the same t and their fields can be compared
            if not mixed:
                L.STS_ARKodeSetFixedStep(I.mem, hseq[k])
            I.evolve(TF, y, sts.ONE_STEP)
            if mixed:
                st = I.stats()
                hseq.append(st["hlast"])
                step_stages.append(st["stages_total"])
        for k in range(args.warmup):
            one_step(k)
        ctx.synchronize()
        barrier()
        s0 = I.stats()
        clocks = Clocks(local)
        clocks.start()
        with timer() as tm:
            for k in range(args.warmup, args.warmup + args.steps):
                one_step(k)
        clock_samples.append(clocks.stop())
        s1 = I.stats()
        ms = max_over_ranks(tm.ms)
        stages = s1["stages_total"] - s0["stages_total"]
        attempts = s1["nst_attempts"] - s0["nst_attempts"]
        dof_stages = N2 * (s1["nfe"] - s0["nfe"])
        stage_ms = I.time_stage_kernel(20)
        kinfo = I.stage_kernel_info()
        kinfo["fusion"] = I.stage_fusion_info()
        # kernels per attempt: stage 1, the stages 2..s (one launch per stage, or per group of
        # ks with a shorter last group), the step end; the timed steps take no rejected attempt
        # here, so the stage counts of the accepted steps are those of the attempts
        ks = kinfo["fusion"]["ks"]
        if ks > 1 and mixed and attempts == args.steps:
            marks = [s0["stages_total"]] + step_stages[args.warmup:]
            launches = sum(step_launches(b - a, ks) for a, b in zip(marks, marks[1:]))
        elif ks > 1:
            launches = attempts * step_launches(stages // attempts if attempts else 0, ks)
        else:
            launches = stages + attempts
        res[mixed] = dict(ms=ms, dof_stages=dof_stages, launches=launches, stage_ms=stage_ms, kinfo=kinfo,
                          t=s1["t"], s=s1["stage_max"], stats=s1, y=y.numpy(), I=I,
                          steps=s1["nst"] - s0["nst"])

    # end to end (mixed): state in from pinned host memory, one step, state back out
    import torch
    I = res[True]["I"]
    # two pinned host buffers in turn: step k reads buffer k % 2 and writes the other, which
    # is the next step's input
    host = [torch.empty(N2, dtype=torch.float64, pin_memory=True) for _ in range(2)]
    host[0].numpy()[:] = res[True]["y"]
    yv = G.vector()
    hp = [C.cast(h.data_ptr(), sts._dp) for h in host]
    t_cur = res[True]["t"]
    k = 0
    for _ in range(2):
        L.N_VCopyFromHost_Sts(yv.h, hp[k])
        I.reset(t_cur, yv)
        t_cur, _ = I.evolve(TF, yv, sts.ONE_STEP)
        L.N_VCopyToHost_Sts(yv.h, hp[1 - k])
        k = 1 - k
    barrier()
    s0 = I.stats()
    clocks = Clocks(local)
    clocks.start()
    with timer() as tm:
        for _ in range(args.steps):
            L.N_VCopyFromHost_Sts(yv.h, hp[k])
            I.reset(t_cur, yv)
            t_cur, _ = I.evolve(TF, yv, sts.ONE_STEP)
            L.N_VCopyToHost_Sts(yv.h, hp[1 - k])
            k = 1 - k
    e2e_clocks = clocks.stop()
    clock_samples.append(e2e_clocks)
    s1 = I.stats()
    e2e_ms = max_over_ranks(tm.ms)
    e2e_stages = (s1["stages_total"] - s0["stages_total"]) / args.steps
    e2e_attempts = s1["nst_attempts"] - s0["nst_attempts"]
    # ARKodeReset evaluates F(t, y) once per step: work of the restart, not of the step
    e2e_dof = N2 * (s1["nfe"] - s0["nfe"] - args.steps)
    # the same calls phase by phase (CUDA events around each, three more steps): where the e2e
    # step goes; the difference to ms_per_step is host time between the calls
    phase = {"h2d": 0.0, "reset": 0.0, "evolve": 0.0, "d2h": 0.0}
    for _ in range(3):
        with timer() as p1:
            L.N_VCopyFromHost_Sts(yv.h, hp[k])
        with timer() as p2:
            I.reset(t_cur, yv)
        with timer() as p3:
            t_cur, _ = I.evolve(TF, yv, sts.ONE_STEP)
        with timer() as p4:
            L.N_VCopyToHost_Sts(yv.h, hp[1 - k])
        k = 1 - k
        for key, tt in zip(phase, (p1, p2, p3, p4)):
            phase[key] += tt.ms / 3
    # the host link alone (copy engine, pinned buffers, same calls): the part of the e2e step
    # that the data dependence between steps keeps from overlapping the device work
    with timer() as th:
        for _ in range(3):
            L.N_VCopyFromHost_Sts(yv.h, hp[k])
    with timer() as td:
        for _ in range(3):
            L.N_VCopyToHost_Sts(yv.h, hp[1 - k])
    h2d_ms, d2h_ms = th.ms / 3, td.ms / 3

    # accuracy on the timed step sequence
    ex = G.exact(res[True]["t"]).numpy()
    out = {}
    for mixed in (True, False):
        yv_ = res[mixed]["y"]
        out[mixed] = float(np.linalg.norm(yv_ - ex) / np.linalg.norm(ex))
    same_t = res[True]["t"] == res[False]["t"]
    if not same_t:
        raise RuntimeError("the FP64 replay of the mixed step sequence ended at another t")
    mix_vs_64 = float(np.linalg.norm(res[True]["y"] - res[False]["y"]) / np.linalg.norm(res[False]["y"]))

    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    m, d = res[True], res[False]
    value = ws * m["dof_stages"] / (m["ms"] / 1e3)
    fp64_value = ws * d["dof_stages"] / (d["ms"] / 1e3)
    # the dominant kernel's algorithmic bytes per launch: one stage reads d_{j-1}, d_{j-2}, F_0
    # and writes d_j (16 B per point); a group of ks stages reads the same three and writes its
    # last two stages (20 B per point for ks stages)
    ks = m["kinfo"]["fusion"]["ks"]
    stage_bytes_mixed = (20.0 if ks > 1 else 16.0) * N2
    stage_bytes_fp64 = 40.0 * N2
    ach = stage_bytes_mixed / (m["stage_ms"] / 1e3) / 1e9
    traffic = fused_stage_traffic(n) if ks > 1 else mixed_stage_traffic(n)
    if ks > 1:
        kdesc = ("mixed stages, %d per launch on 120x%d shared-memory tiles (20 B per point and launch, "
                 "%.1f B/DOF-stage): %s" % (ks, m["kinfo"]["fusion"]["tile_rows"], 20.0 / ks, m["kinfo"]["name"]))
    else:
        kdesc = "mixed stage kernel (16 B/DOF-stage), autotuned: %s" % m["kinfo"]["name"]
    fp64_flops = 17.0 * N2 / (d["stage_ms"] / 1e3)
    fp64_peak = C.c_double()
    fp64_peak_tflops = fp64_peak.value if sts.lib().STS_ProbeFP64Rate(ctx.h, C.byref(fp64_peak)) == 0 else None
    line = {
        "metric": "STS DOF-stages/s & solve time at 8192^2: mixed vs FP64 GPU at 1e-6 rel L2 err",
        "value": value,
        "unit": "DOF-stages/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": m["ms"] / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 stage increments + f64 step update",
        "data": "synthetic (manufactured-solution initial state, no dataset)",
        "config": {"workload": "manufactured 2-D heat %dx%d, kx=1 ky=1e-2, RKL2 adaptive, rtol=1e-6 "
                               "atol=1e-10, smax=200, t in [0,0.05]" % (n, n),
                   "nx": n, "ny": n, "method": "RKL2", "stages_per_step": m["s"],
                   "inputs_exceed_l2": True, "parallelism": "replicas" if ws > 1 else "single GPU"},
        "e2e": {"value": ws * e2e_dof / (e2e_ms / 1e3), "unit": "DOF-stages/s",
                "h2d_bytes_per_step": 8 * N2, "d2h_bytes_per_step": 8 * N2,
                "ms_per_step": e2e_ms / args.steps, "h2d_ms": h2d_ms, "d2h_ms": d2h_ms,
                "h2d_gbs": 8 * N2 / (h2d_ms / 1e3) / 1e9, "d2h_gbs": 8 * N2 / (d2h_ms / 1e3) / 1e9,
                "stages_per_step": e2e_stages, "step_attempts": e2e_attempts, "sm_mhz": e2e_clocks["sm_mhz"],
                "phase_ms": {q: round(v, 3) for q, v in phase.items()}},
        "gpu_launches": m["launches"],
        "roofline": {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                     "frac": ach / peak, "traffic": traffic, "kernel": kdesc,
                     "ms_per_launch": m["stage_ms"], "dof_stages_per_launch": ks * N2,
                     "kernel_dof_stages_per_s": ks * N2 / (m["stage_ms"] / 1e3),
                     # the DOF-stage rate against the HBM bound of one launch per stage
                     # (16 B per DOF-stage at the same peak): above 1 only with stage groups
                     "vs_single_stage_hbm_bound": (ks * N2 / (m["stage_ms"] / 1e3)) / (peak * 1e9 / 16.0),
                     "peak_source": peak_kind},
        "clocks": merge_clocks(clock_samples),
        "fp64": {"value": fp64_value, "unit": "DOF-stages/s", "ms_per_step": d["ms"] / args.steps,
                 "stage_kernel_ms": d["stage_ms"],
                 "stage_kernel_hbm_gbs": stage_bytes_fp64 / (d["stage_ms"] / 1e3) / 1e9,
                 "stage_kernel_fp64_tflops": fp64_flops / 1e12,
                 "fp64_peak_tflops_probed": fp64_peak_tflops,
                 "stage_kernel_fp64_frac": (fp64_flops / 1e12 / fp64_peak_tflops) if fp64_peak_tflops else None,
                 "fp64_peak_note": "FP64 FMA rate probed in this run (STS_ProbeFP64Rate: independent FMA "
                                   "chains, 8 blocks per SM); the stage kernel does 17 flops per DOF-stage"},
        "speedup_mixed_vs_fp64": value / fp64_value,
        "accuracy": {"t": m["t"], "mixed_rel_l2_vs_exact": out[True], "fp64_rel_l2_vs_exact": out[False],
                     "mixed_vs_fp64_rel_l2": mix_vs_64},
    }
    cpu = cpu_baseline(args) if not args.no_cpu else None
    line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)


def cpu_step_setup(n, stages):
    """Oracle integrator at n^2 with a fixed step that needs exactly `stages` RKL2 stages."""
    from oracle import pyoracle as po
    P = po.Problem(po.MANUFACTURED, n, n, kx=KX, ky=KY)
    rho = 1.01 * abs(P.dom_eig())
    s = stages
    h = (s * s + s - 2) / (2.0 * rho) * 0.999
    I = po.Integrator(P, P.initial(), method=po.RKL, rtol=RTOL, atol=ATOL, hfixed=h, maxsteps=1)
    return po, P, I, h


def cpu_baseline(args, stages=196, nsteps=2):
    """A bounded sample of the workload on the CPU oracle: `nsteps` fixed RKL2 steps of
    `stages` stages (the stage count of the timed GPU steps) after one untimed step."""
    po, P, I, h = cpu_step_setup(args.n, stages)
    I.evolve(TF)  # initialisation + first step (untimed)
    s0 = I.stats()
    t0 = time.perf_counter()
    for _ in range(nsteps):
        I.evolve(TF)
    dt = time.perf_counter() - t0
    s1 = I.stats()
    dof = args.n * args.n * (s1["nfe"] - s0["nfe"])
    return {"value": dof / dt, "unit": "DOF-stages/s", "cores": po.lib().orc_nthreads(),
            "kind": "port",
            "sample": "%d fixed-step RKL2 steps (%d RHS evaluations) of the %d^2 FP64 problem on the "
                      "CPU oracle" % (nsteps, s1["nfe"] - s0["nfe"], args.n)}


def run_reference(args):
    """The reference algorithm on the host cores (the CPU oracle, FP64, all threads) on the
    same workload as the GPU arm: adaptive RKL2 from t = 0 (rtol 1e-6, atol 1e-10, at most
    200 stages), `warmup` untimed steps, then `steps` timed steps."""
    ws, rank, local = dist_info()
    if rank != 0:
        return
    from oracle import pyoracle as po
    n = args.n
    P = po.Problem(po.MANUFACTURED, n, n, kx=KX, ky=KY)
    I = po.Integrator(P, P.initial(), method=po.RKL, rtol=RTOL, atol=ATOL, smax=SMAX, maxsteps=1)
    for _ in range(args.warmup):
        I.evolve(TF)
    s0 = I.stats()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        I.evolve(TF)
    dt = time.perf_counter() - t0
    s1 = I.stats()
    dof = n * n * (s1["nfe"] - s0["nfe"])
    v = dof / dt
    sample = ("%d adaptive RKL2 steps (after %d untimed) of the %d^2 FP64 problem, %d RHS evaluations; "
              "CPU restatement of the reference algorithm (SUNDIALS is not vendored in the reference, "
              "so the reference binary cannot be built)" % (args.steps, args.warmup, n,
                                                            s1["nfe"] - s0["nfe"]))
    line = {
        "metric": "STS DOF-stages/s & solve time at 8192^2: mixed vs FP64 GPU at 1e-6 rel L2 err",
        "value": v, "unit": "DOF-stages/s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (manufactured-solution initial state)",
        "config": {"workload": "manufactured 2-D heat %dx%d, kx=1 ky=1e-2, RKL2 adaptive, rtol=1e-6 "
                               "atol=1e-10, smax=200, t in [0,0.05]" % (n, n),
                   "nx": n, "ny": n, "method": "RKL2", "stages_per_step": s1["stage_max"],
                   "t_end_of_timed_steps": s1["t"]},
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": "DOF-stages/s", "cores": po.lib().orc_nthreads(),
                         "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "DOF-stages/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_full(args):
    """Time-to-solution on [0, tf] for both precisions (one run each per method / rtol)."""
    import numpy as np
    import ceda_demonstrations_gb300 as sts
    ctx = sts.Context(0)
    timer = cuda_timer(ctx.stream)
    n, tf, kx, ky = args.n, args.tf, args.kx, args.ky
    G = sts.Problem(ctx, sts.MANUFACTURED, n, n, kx, ky)
    ex = G.exact(tf).numpy()
    out = {}
    methods = [1, 0] if args.both_methods else [1]
    rtols = [1e-6, 1e-4] if args.both_rtols else [1e-6]
    for method in methods:
        for rtol in rtols:
            ys = {}
            for mixed in (True, False):
                I = sts.LSRKStep(ctx, G, 0.0, G.initial(), method=method, rtol=rtol, atol=ATOL,
                                 smax=SMAX, mixed=mixed, graphs=True, maxsteps=1000000)
                I.set_stop_time(tf)  # the last step ends on tf (diffusion_2D/main.cpp:384)
                y = G.vector()
                with timer() as tm:
                    I.evolve(tf, y)
                st = I.stats()
                ys[mixed] = y.numpy()
                key = "%s_rtol%g_%s" % ("RKL2" if method else "RKC2", rtol, "mixed" if mixed else "fp64")
                out[key] = {"time_to_solution_s": tm.ms / 1e3, "steps": st["nst"], "netf": st["netf"],
                            "rhs_evals": st["nfe"], "stage_max": st["stage_max"],
                            "dof_stages_per_s": n * n * st["nfe"] / (tm.ms / 1e3),
                            "rel_l2_vs_exact": float(np.linalg.norm(ys[mixed] - ex) / np.linalg.norm(ex))}
                print(key, json.dumps(out[key]), flush=True)
                I.free()
            rel = float(np.linalg.norm(ys[True] - ys[False]) / np.linalg.norm(ys[False]))
            tag = "%s_rtol%g" % ("RKL2" if method else "RKC2", rtol)
            out[tag + "_mixed_vs_fp64_rel_l2"] = rel
            out[tag + "_speedup"] = out[tag + "_fp64"]["time_to_solution_s"] / out[tag + "_mixed"]["time_to_solution_s"]
            print(tag, "mixed vs fp64 rel L2", rel, "speedup", out[tag + "_speedup"], flush=True)
    print(json.dumps({"full_solve": out, "n": n, "tf": tf, "kx": kx, "ky": ky}), flush=True)


def run_config1(args):
    """The serial CPU configuration (128^2, kx = ky = 1, manufactured problem, RKC adaptive,
    rtol 1e-6, atol 1e-10, t in [0, 1], stop time 1): time to solution of the FP64 GPU path
    (CUDA events around the evolve) and of the CPU oracle on one thread (the reference's serial
    single-rank run) and on all host threads, with the final fields compared."""
    import numpy as np
    import ceda_demonstrations_gb300 as sts
    from oracle import pyoracle as po
    ctx = sts.Context(0)
    timer = cuda_timer(ctx.stream)
    n, tf = 128, 1.0
    G = sts.Problem(ctx, sts.MANUFACTURED, n, n, 1.0, 1.0)
    out = {}
    for rep in range(2):  # the first run warms up the graphs and the autotuner
        I = sts.LSRKStep(ctx, G, 0.0, G.initial(), method=sts.RKC, rtol=1e-6, atol=1e-10, maxsteps=10 ** 6)
        I.set_stop_time(tf)
        y = G.vector()
        with timer() as tm:
            I.evolve(tf, y)
        st = I.stats()
        yg = y.numpy()
        I.free()
    ex = G.exact(tf).numpy()
    out["gpu"] = {"seconds": tm.ms / 1e3, "steps": st["nst"], "rhs_evals": st["nfe"],
                  "rel_l2_vs_exact": float(np.linalg.norm(yg - ex) / np.linalg.norm(ex))}
    P = po.Problem(po.MANUFACTURED, n, n, kx=1.0, ky=1.0)
    allt = po.lib().orc_nthreads()
    for label, nth in (("cpu_1_thread", 1), ("cpu_all_threads", allt)):
        po.lib().orc_set_nthreads(nth)
        J = po.Integrator(P, P.initial(), method=po.RKC, rtol=1e-6, atol=1e-10, maxsteps=10 ** 6, tstop=tf)
        t0 = time.perf_counter()
        J.evolve(tf)
        sec = time.perf_counter() - t0
        out[label] = {"seconds": sec, "threads": nth, "steps": J.stats()["nst"],
                      "same_bits_as_gpu": bool(np.array_equal(J.y, yg))}
    po.lib().orc_set_nthreads(allt)
    out["gpu_speedup_vs_1_thread"] = out["cpu_1_thread"]["seconds"] / out["gpu"]["seconds"]
    print(json.dumps({"config1": out, "n": n, "tf": tf}), flush=True)


def run_reference_mode(args):
    """The reference's own problem (periodic, Gaussian x sine initial state, inhomogeneous
    faces k (1 + 0.99 sin)) at 2048^2, RKL2 rtol 1e-5: FP64 and mixed reference mode from
    t = 0.01 (untimed) to t = 0.05 (timed, CUDA events), DOF-stages/s of each."""
    import numpy as np
    import ceda_demonstrations_gb300 as sts
    ctx = sts.Context(0)
    timer = cuda_timer(ctx.stream)
    n = args.refmode_n
    out = {}
    ys = {}
    for mixed in (False, True):
        G = sts.Problem(ctx, sts.PERIODIC, n, n, 1.0, 1.0, inhomogeneous=True)
        I = sts.LSRKStep(ctx, G, 0.0, G.initial(), method=sts.RKL, rtol=1e-5, atol=1e-9, mixed=mixed,
                         maxsteps=1000000)
        y = G.vector()
        I.evolve(0.01, y)
        ctx.synchronize()
        s0 = I.stats()
        I.set_stop_time(0.05)
        with timer() as tm:
            I.evolve(0.05, y)
        s1 = I.stats()
        dof = n * n * (s1["nfe"] - s0["nfe"])
        key = "mixed" if mixed else "fp64"
        out[key] = {"seconds": tm.ms / 1e3, "steps": s1["nst"] - s0["nst"], "rhs_evals": s1["nfe"] - s0["nfe"],
                    "stage_max": s1["stage_max"], "dof_stages_per_s": dof / (tm.ms / 1e3)}
        ys[mixed] = y.numpy()
        print(key, json.dumps(out[key]), flush=True)
        I.free()
    rel = float(np.linalg.norm(ys[True] - ys[False]) / np.linalg.norm(ys[False]))
    print(json.dumps({"reference_mode": out, "n": n, "mixed_vs_fp64_rel_l2_adaptive": rel,
                      "speedup": out["fp64"]["seconds"] / out["mixed"]["seconds"]}), flush=True)


def run_batch_profile(args):
    """A small batch for counter captures: `--batch-count` seeded instances, a fixed launch
    shape (256 threads, 4 CTAs/SM, 8-CTA clusters for n >= 256: the autotuner's usual choice),
    one FP64 evolve and one mixed evolve to `--batch-tf`. Prints the DOF-stages and DOF-steps
    of each (the per-launch normalisation of the counters) and the time of each evolve."""
    import ceda_demonstrations_gb300 as sts
    ctx = sts.Context(0)
    inst = sts.make_batch_instances(count=args.batch_count, seed=20261203)
    res = {}
    for mixed in (False, True):
        B = sts.Batch(ctx, inst)
        B.set_mixed(mixed)
        B.set_launch(256, 4, 8, 256)
        B.evolve(args.batch_tf, method=sts.RKL, rtol=1e-6, atol=1e-10, smax=SMAX)  # warm-up
        B2 = sts.Batch(ctx, inst)
        B2.set_mixed(mixed)
        B2.set_launch(256, 4, 8, 256)
        ms = B2.evolve(args.batch_tf, method=sts.RKL, rtol=1e-6, atol=1e-10, smax=SMAX)
        st = [B2.stats(i) for i in range(len(inst))]
        dof_stages = sum(inst[i][0] ** 2 * st[i]["nfe"] for i in range(len(inst)))
        dof_steps = sum(inst[i][0] ** 2 * st[i]["nst_attempts"] for i in range(len(inst)))
        res["mixed" if mixed else "fp64"] = {
            "ms": ms, "dof_stages": dof_stages, "dof_step_attempts": dof_steps,
            "stages_per_step": dof_stages / dof_steps, "dof_stages_per_s": dof_stages / (ms / 1e3),
            "largest_instance_share": max(inst[i][0] ** 2 * st[i]["nfe"] for i in range(len(inst))) / dof_stages,
            "sizes": sorted(set(int(x[0]) for x in inst))}
        B.free()
        B2.free()
    print(json.dumps({"batch_profile": res, "count": len(inst), "tf": args.batch_tf}), flush=True)


def run_batch(args):
    """512 independent heat problems in one persistent launch (n uniform from
    {64,...,512}, kx, ky log-uniform in [1e-2, 1], 8 random sine modes, RKL2 rtol 1e-6 to
    t = 0.01, per-instance step control on the device)."""
    import numpy as np
    import ceda_demonstrations_gb300 as sts
    from oracle import pyoracle as po
    ctx = sts.Context(0)
    inst = sts.make_batch_instances(count=args.batch_count, seed=20261203)
    B = sts.Batch(ctx, inst)
    th, cp, tune_ms = B.autotune(0.25 * args.batch_tf)
    ms = B.evolve(args.batch_tf, method=sts.RKL, rtol=1e-6, atol=1e-10, smax=SMAX)
    y = B.state()
    nfe = [B.stats(i)["nfe"] for i in range(len(inst))]
    nst = [B.stats(i)["nst"] for i in range(len(inst))]
    dof_stages = float(sum(inst[i][0] ** 2 * nfe[i] for i in range(len(inst))))
    per_inst = sorted((inst[i][0] ** 2 * nfe[i] for i in range(len(inst))), reverse=True)
    # CPU oracle on a sample of instances (all host threads), and parity on that sample
    sample = list(range(0, len(inst), max(1, len(inst) // 16)))[:16]
    t0 = time.perf_counter()
    cpu_dof = 0.0
    maxrel = 0.0
    for i in sample:
        n, kx, ky, p, q, a = inst[i]
        P = po.Problem(po.UNFORCED, n, n, kx=kx, ky=ky)
        J = po.Integrator(P, P.initial_modes(p, q, a), method=po.RKL, rtol=1e-6, atol=1e-10,
                          tstop=args.batch_tf)  # the batch ends every instance on tf
        J.evolve(args.batch_tf)
        cpu_dof += n * n * J.stats()["nfe"]
        yi = B.instance_state(y, i)
        maxrel = max(maxrel, float(np.linalg.norm(yi - J.y) / np.linalg.norm(J.y)))
    cpu_s = time.perf_counter() - t0
    # the same batch with FP32 stage increments (own autotune), parity against the oracle's
    # mixed integrator on the sample and accuracy against the FP64 batch
    M = sts.Batch(ctx, inst)
    M.set_mixed(True)
    mth, mcp, mtune = M.autotune(0.25 * args.batch_tf)
    mms = M.evolve(args.batch_tf, method=sts.RKL, rtol=1e-6, atol=1e-10, smax=SMAX)
    ym = M.state()
    mnfe = [M.stats(i)["nfe"] for i in range(len(inst))]
    mdof = float(sum(inst[i][0] ** 2 * mnfe[i] for i in range(len(inst))))
    mmax_or, mmax_64 = 0.0, 0.0
    for i in sample:
        n, kx, ky, p, q, a = inst[i]
        P = po.Problem(po.UNFORCED, n, n, kx=kx, ky=ky)
        J = po.Integrator(P, P.initial_modes(p, q, a), method=po.RKL, rtol=1e-6, atol=1e-10,
                          mixed=True, tstop=args.batch_tf)
        J.evolve(args.batch_tf)
        yi = M.instance_state(ym, i)
        mmax_or = max(mmax_or, float(np.linalg.norm(yi - J.y) / np.linalg.norm(J.y)))
    for i in range(len(inst)):
        ref = B.instance_state(y, i)
        mmax_64 = max(mmax_64, float(np.linalg.norm(M.instance_state(ym, i) - ref) / np.linalg.norm(ref)))
    line = {
        "metric": "batched STS: DOF-stages/s and time for %d independent problems in one launch" % len(inst),
        "value": dof_stages / (ms / 1e3), "unit": "DOF-stages/s", "time_s": ms / 1e3,
        "total_dof": int(B.total), "dof_stages": dof_stages, "steps_total": int(sum(nst)),
        "steps_max": int(max(nst)),
        "launch": {"threads": th, "ctas_per_sm": cp, "cluster_large": B.launch()[2],
                   "cluster_min_n": B.launch()[3], "probe_ms": tune_ms},
        "largest_instance_dof_stages": float(per_inst[0]),
        "largest_instance_share": float(per_inst[0]) / dof_stages,
        "dtype": "f64", "data": "synthetic (seeded sine-mode initial states, seed 20261203)",
        "parity_sample_max_rel_l2_vs_oracle": maxrel,
        "mixed": {"value": mdof / (mms / 1e3), "unit": "DOF-stages/s", "time_s": mms / 1e3,
                  "dof_stages": mdof, "speedup_vs_f64": (mdof / (mms / 1e3)) / (dof_stages / (ms / 1e3)),
                  "launch": {"threads": mth, "ctas_per_sm": mcp, "cluster_large": M.launch()[2],
                             "probe_ms": mtune},
                  "parity_sample_max_rel_l2_vs_mixed_oracle": mmax_or,
                  "max_rel_l2_vs_f64_batch": mmax_64,
                  "dtype": "f32 stage increments + f64 step update"},
        "cpu_baseline": {"value": cpu_dof / cpu_s, "unit": "DOF-stages/s", "cores": po.lib().orc_nthreads(),
                         "kind": "port", "sample": "%d of the %d instances, integrated one after another"
                                                   % (len(sample), len(inst))},
    }
    print(json.dumps(line), flush=True)


def run_precond(args):
    """Implicit comparator with the learned preconditioner on 2048^2 shifted systems
    (I - gamma_h A) x = r: kx = 1, ky log-uniform in [1e-3, 1], gamma_h log-uniform in
    [1e-4, 1e-2], r a seeded random smooth field. Training pairs come from Jacobi-PCG solves
    of other seeded systems (crops of r_k and e_k = x* - x_k); the network is trained on
    the GPU; the evaluation solves unseen systems to a 1e-8 relative FP64 residual with FCG
    + network and with Jacobi-PCG and compares their wall times."""
    import numpy as np
    import torch
    import ceda_demonstrations_gb300 as sts
    ctx = sts.Context(0)
    n, crop = args.precond_n, args.precond_crop
    dx = 1.0 / (n + 1)
    rng = np.random.default_rng(20261203)

    def system(rng):
        ky = 10.0 ** rng.uniform(-3.0, 0.0)
        gh = 10.0 ** rng.uniform(-4.0, -2.0)
        return ky, gh

    # 1. training pairs
    cap = args.precond_pairs
    r_all = torch.empty(cap * crop * crop, dtype=torch.float32, device="cuda")
    e_all = torch.empty_like(r_all)
    meta = torch.empty(cap * 7, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    got, nsys, pcg_its = 0, 0, []
    while got < cap and nsys < 400:
        ky, gh = system(rng)
        P = sts.Problem(ctx, sts.UNFORCED, n, n, 1.0, ky)
        b = sts.NVector.from_numpy(ctx, sts.smooth_field(n, rng))
        off = got * crop * crop
        k, its = sts.harvest_pcg_pairs(P, gh, b, args.precond_crops, crop, args.precond_every,
                                       min(cap - got, 4000), r_all.data_ptr() + 4 * off,
                                       e_all.data_ptr() + 4 * off, meta.data_ptr() + 4 * 7 * got,
                                       int(rng.integers(1 << 62)))
        got += k
        nsys += 1
        pcg_its.append(its)
        P.free()
        b.destroy()
    torch.cuda.synchronize()
    harvest_s = time.perf_counter() - t0
    # 2. training
    net = sts.Net(ctx, n, seed=1)
    t0 = time.perf_counter()
    losses = []
    for ep, lr in enumerate([2e-3] * (args.precond_epochs // 2) + [7e-4] * (args.precond_epochs // 4)
                            + [2e-4] * (args.precond_epochs - args.precond_epochs // 2 - args.precond_epochs // 4)):
        losses.append(net.train(crop, got, r_all.data_ptr(), e_all.data_ptr(), meta.data_ptr(), 1,
                                args.precond_batch, lr, seed=ep))
    train_s = time.perf_counter() - t0
    del r_all, e_all, meta
    torch.cuda.empty_cache()
    # 3. evaluation on unseen systems
    erng = np.random.default_rng(777)
    rows = []
    for k in range(args.precond_eval):
        ky, gh = system(erng)
        P = sts.Problem(ctx, sts.UNFORCED, n, n, 1.0, ky)
        b = sts.NVector.from_numpy(ctx, sts.smooth_field(n, erng))
        x1, x2, x3, x4 = P.vector(), P.vector(), P.vector(), P.vector()
        mg = sts.PFMG(P, relax=2, nrelax=2)  # the reference's multilevel comparator (PFMG role)
        # the network behind PSetup / PSolve inside flexible GMRES(30), classical Gram-Schmidt
        NP = sts.NetPrec(net, P)
        FG = sts.SPFGMRSolver(ctx, b, maxl=30, max_restarts=2000, gstype=sts.CLASSICAL_GS, precond=True)
        res = {}
        for rep in range(2):  # the first solve of each kind warms up (graph instantiation)
            ctx.synchronize()
            t = time.perf_counter()
            it1, rel1, rc1 = sts.implicit_solve_pcg(P, gh, b, x1, tol=1e-8, maxit=200000)
            t_pcg = time.perf_counter() - t
            ctx.synchronize()
            t = time.perf_counter()
            it2, rel2, rc2 = sts.fcg_solve(P, gh, net, b, x2, tol=1e-8, maxit=20000)
            t_fcg = time.perf_counter() - t
            ctx.synchronize()
            t = time.perf_counter()
            it3, rel3, rc3, used = sts.implicit_solve_learned(P, gh, net, b, x2, tol=1e-8, maxit=20000)
            t_auto = time.perf_counter() - t
            ctx.synchronize()
            t = time.perf_counter()
            it4, rel4, rc4 = sts.implicit_solve_pfmg(P, gh, mg, b, x3, tol=1e-8, maxit=10000)
            t_mg = time.perf_counter() - t
            ctx.synchronize()
            t = time.perf_counter()
            NP.setup(gh)
            rc5, it5, rel5 = sts.implicit_solve_ls(P, gh, FG, b, x4, tol=1e-8, prec=sts.PREC_USER,
                                                   pdata=NP.h, psolve=NP.psolve_fn)
            t_fg = time.perf_counter() - t
            res = {"ky": ky, "gamma_h": gh, "pcg_iters": it1, "pcg_s": t_pcg, "pcg_relres": rel1,
                   "fgmres_net_iters": it5, "fgmres_net_s": t_fg, "fgmres_net_relres": rel5,
                   "fgmres_net_status": rc5,
                   "pfmg_iters": it4, "pfmg_s": t_mg, "pfmg_relres": rel4, "pfmg_levels": mg.levels(),
                   "fcg_iters": it2, "fcg_s": t_fcg, "fcg_true_relres": rel2, "fcg_status": rc2,
                   "pcg_ms_per_iter": 1e3 * t_pcg / max(1, it1),
                   "fcg_ms_per_iter": 1e3 * t_fcg / max(1, it2),
                   "learned_s": t_auto, "learned_used_net": used, "learned_iters": it3,
                   "learned_relres": rel3}
        xa, xb = x1.numpy(), x2.numpy()
        res["solution_rel_diff"] = float(np.linalg.norm(xa - xb) / np.linalg.norm(xa))
        res["pfmg_solution_rel_diff"] = float(np.linalg.norm(xa - x3.numpy()) / np.linalg.norm(xa))
        res["fgmres_net_solution_rel_diff"] = float(np.linalg.norm(xa - x4.numpy()) / np.linalg.norm(xa))
        rows.append(res)
        print(json.dumps(res), flush=True)
        del mg, FG, NP
        P.free()
    t_pcg = sum(r["pcg_s"] for r in rows)
    t_fcg = sum(r["fcg_s"] for r in rows)
    t_auto = sum(r["learned_s"] for r in rows)
    line = {
        "metric": "implicit solve wall time, Jacobi-PCG / learned-preconditioner solve "
                  "(STS_ImplicitSolveLearned), 1e-8 rel residual, %d^2" % n,
        "value": t_pcg / t_auto, "unit": "x", "higher_is_better": True, "n_gpus": 1,
        "pcg_total_s": t_pcg, "learned_total_s": t_auto, "fcg_total_s": t_fcg,
        "fcg_only_speedup": t_pcg / t_fcg,
        "pfmg_total_s": sum(r["pfmg_s"] for r in rows),
        "pfmg_speedup_vs_jacobi_pcg": t_pcg / max(1e-12, sum(r["pfmg_s"] for r in rows)),
        "fgmres_net_total_s": sum(r["fgmres_net_s"] for r in rows),
        "fgmres_net_speedup_vs_jacobi_pcg": t_pcg / max(1e-12, sum(r["fgmres_net_s"] for r in rows)),
        "systems_on_net": sum(1 for r in rows if r["learned_used_net"]),
        "max_learned_relres": max(r["learned_relres"] for r in rows),
        "iters_ratio": sum(r["pcg_iters"] for r in rows) / max(1, sum(r["fcg_iters"] for r in rows)),
        "max_fcg_true_relres": max(r["fcg_true_relres"] for r in rows),
        "training": {"pairs": got, "crop": crop, "systems": nsys, "harvest_s": harvest_s,
                     "train_s": train_s, "epochs": args.precond_epochs, "batch": args.precond_batch,
                     "loss_first_epoch": losses[0] if losses else None,
                     "loss_last_epoch": losses[-1] if losses else None,
                     "pcg_iters_mean": float(np.mean(pcg_its))},
        "dtype": "bf16 net (fp32 accumulate), f64 Krylov",
        "data": "synthetic (seeded smooth right-hand sides, seed 20261203 / 777)",
        "config": {"workload": "(I - gamma_h A) x = r, %d^2, kx=1, ky log-uniform [1e-3,1], gamma_h "
                               "log-uniform [1e-4,1e-2]" % n, "eval_systems": len(rows)},
    }
    print(json.dumps(line), flush=True)


def run_precond_profile(args):
    """A short FCG + network solve and a short Jacobi-PCG solve on one 2048^2 system (16
    iterations each, untrained network), for kernel launch lists."""
    import numpy as np
    import ceda_demonstrations_gb300 as sts
    ctx = sts.Context(0)
    n = args.precond_n
    rng = np.random.default_rng(5)
    P = sts.Problem(ctx, sts.UNFORCED, n, n, 1.0, 0.1)
    b = sts.NVector.from_numpy(ctx, sts.smooth_field(n, rng))
    x = P.vector()
    net = sts.Net(ctx, n, seed=1)
    gh = 1e-3
    # tolerances no solve reaches in 16 iterations; FCG without its fallback (negative maxit)
    for _ in range(args.warmup):
        sts.fcg_solve(P, gh, net, b, x, tol=1e-14, maxit=-16)
        sts.implicit_solve_pcg(P, gh, b, x, tol=1e-14, maxit=16)
    ctx.synchronize()
    t0 = time.perf_counter()
    it1, _, _ = sts.fcg_solve(P, gh, net, b, x, tol=1e-14, maxit=-16)
    t1 = time.perf_counter()
    it2, _, _ = sts.implicit_solve_pcg(P, gh, b, x, tol=1e-14, maxit=16)
    t2 = time.perf_counter()
    print(json.dumps({"fcg_iters": it1, "fcg_ms_per_iter": 1e3 * (t1 - t0) / max(1, it1),
                      "pcg_iters": it2, "pcg_ms_per_iter": 1e3 * (t2 - t1) / max(1, it2)}), flush=True)


def run_net_apply(args):
    """One application of the (untrained) network at 2048^2 on each inference path: the
    convolutions of levels 1-3 on mma.sync (0) or on tcgen05 + TMEM (1), level 0 collapsed in
    both; CUDA events over 50 applications after 5 untimed ones."""
    import numpy as np
    import ceda_demonstrations_gb300 as sts
    ctx = sts.Context(0)
    timer = cuda_timer(ctx.stream)
    n = args.precond_n
    rng = np.random.default_rng(5)
    net = sts.Net(ctx, n, seed=1)
    rv = sts.NVector.from_numpy(ctx, sts.smooth_field(n, rng))
    zv = sts.NVector(ctx, n * n)
    out = {}
    for path in (0, 1):
        net.set_tensor_path(path)
        for _ in range(5):
            net.apply(n, rv.ptr, zv.ptr, 0.3, -0.2, 0.5, 1.0)
        ctx.synchronize()
        with timer() as t:
            for _ in range(50):
                net.apply(n, rv.ptr, zv.ptr, 0.3, -0.2, 0.5, 1.0)
        out["mma_sync" if path == 0 else "tcgen05"] = {"us_per_application": t.ms / 50 * 1e3}
    net.set_tensor_path(0)
    print(json.dumps({"net_apply": out, "n": n}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--full", action="store_true")
    ap.add_argument("--tf", type=float, default=TF)
    ap.add_argument("--kx", type=float, default=KX)
    ap.add_argument("--ky", type=float, default=KY)
    ap.add_argument("--both-methods", action="store_true")
    ap.add_argument("--both-rtols", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--stage-fusion", type=int, default=0,
                    help="mixed stages per launch: 0 autotuned, 1 off, 2-4 (STS_LSRKStepSetStageFusion)")
    ap.add_argument("--fusion-config", type=int, default=0,
                    help="fused tile configuration: 0 autotuned, 1-4 (STS_LSRKStepSetStageFusion)")
    ap.add_argument("--stage-kernel", type=int, default=0,
                    help="mixed stage kernel: 0 autotune, 1 register marching, 2+k TMA configuration k")
    ap.add_argument("--reference-mode", action="store_true")
    ap.add_argument("--config1", action="store_true")
    ap.add_argument("--refmode-n", type=int, default=2048)
    ap.add_argument("--batch", action="store_true")
    ap.add_argument("--batch-profile", action="store_true")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--batch-tf", type=float, default=0.01)
    ap.add_argument("--precond", action="store_true")
    ap.add_argument("--precond-profile", action="store_true")
    ap.add_argument("--net-apply", action="store_true")
    ap.add_argument("--precond-n", type=int, default=2048)
    ap.add_argument("--precond-crop", type=int, default=128)
    ap.add_argument("--precond-crops", type=int, default=4)
    ap.add_argument("--precond-every", type=int, default=1)
    ap.add_argument("--precond-pairs", type=int, default=102400)
    ap.add_argument("--precond-epochs", type=int, default=24)
    ap.add_argument("--precond-batch", type=int, default=32)
    ap.add_argument("--precond-eval", type=int, default=8)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.full:
        run_full(args)
    elif args.reference_mode:
        run_reference_mode(args)
    elif args.config1:
        run_config1(args)
    elif args.batch_profile:
        run_batch_profile(args)
    elif args.batch:
        run_batch(args)
    elif args.precond:
        run_precond(args)
    elif args.precond_profile:
        run_precond_profile(args)
    elif args.net_apply:
        run_net_apply(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
