#!/usr/bin/env python
"""Headline benchmark: member-steps/s of the ensemble pipe-flow stepper on GB300.

Workload (the batched-ensemble configuration the metric is quoted on): 64
independent pipes of the NR=48, 32 x 64-mode size (NR=48, NT=32, NZ=65), Re_b=2000,
L=4piR (LZ = 2*2pi), dt = 0.005 R/U_b (0.01 code units), each from Hagen-Poiseuille
flow plus its own seeded divergence-free perturbation of amplitude
1e-3 (1 + 0.01 i), seed 2000 + i.  One step = one full predictor-corrector time
step of every member (the reference's integrate() loop body), corrector
iterations to tol = 5e-8 as in the reference.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64]
    python bench.py --impl reference ...   # the reference nsPipe-CUDA build, same workload
    python bench.py --workload uneven      # the uneven batch alone: 28 pipes of three resolutions, mixed

The headline line also carries the plain FP64 form on the same ensemble (device-timed
and end to end) and the uneven batch as sub-objects.  Under torchrun each rank (one
GPU) advances its own 64-member ensemble (weak scaling, no data-path collective), or
with --split its shard of one 64-member ensemble (strong scaling); timing is bracketed
by a barrier and synchronisation and the max over ranks is taken.  Rank 0 prints one
JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "nspipe-gpu_gb300"))

METRIC = "member-steps/s and ns/(step·dof), mixed+batched vs plain FP64 on 1 GB300"
UNIT = "member-steps/s"
PI2 = 6.283185307179586
NR, NT, NZ, RE, DT, LZ = 48, 32, 65, 2000.0, 0.01, 2.0 * PI2
MEMBERS = 64
S = NR * NT * NZ
DOF = 3 * S
WORKLOAD = "ensemble of 64 pipes NR=48 x 32 theta x 64 axial modes (NT=32, NZ=65), Re_b=2000, L=4piR, dt=0.005R/U_b"


def member_fields(m, seed_base=2000):
    from nspipe_gb300 import seeded_field
    return seeded_field(NR, NT, NZ, LZ, 1e-3 * (1.0 + 0.01 * m), seed_base + m)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        # Start timing only once nvidia-smi is sampling: its start-up (NVML
        # initialisation on a fresh machine) must not overlap the timed steps.
        t0 = time.time()
        while self.proc and time.time() - t0 < 10.0:
            try:
                if os.path.getsize(self.path) > 0:
                    break
            except OSError:
                pass
            time.sleep(0.05)
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=10)

    def summary(self):
        rows = []
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) >= 8 and f[0].replace(".", "").isdigit():
                    rows.append(f)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[0]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[4 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": float(rows[0][1]), "reasons": reasons,
                "samples": len(rows), "power_w_max": max(float(r[2]) for r in rows if r[2][:1].isdigit())}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ------------------------------------------------------------------ CPU baseline (oracle port)
def cpu_baseline(budget_s=12.0):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    cores = os.cpu_count() or 1
    o = oracle.Oracle(NR, NT, NZ, Re=RE, dt=DT, LZ=LZ, nthreads=cores)
    u = member_fields(0)
    u, _, _ = o.step(u, 1)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s and steps < 200:
        u, _, _ = o.step(u, 1)
        steps += 1
    el = time.perf_counter() - t0
    o.close()
    return {"value": steps / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "1 member of the workload, %d time steps, FP64 C restatement (oracle/), OpenMP %d threads"
                      % (steps, cores)}


# ------------------------------------------------------------------ reference arm
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
    import build_ref
    steps_per_sample = 20
    line = {"impl": "reference", "metric": METRIC, "unit": UNIT, "higher_is_better": True, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup}
    try:
        build_ref.build("c0", "time", nsteps=steps_per_sample)
    except Exception as e:  # sources not staged or no compiler
        line["unavailable"] = "reference build failed: %s" % str(e).splitlines()[0][:200]
        print(json.dumps(line))
        return 0
    from nspipe_gb300.initfield import write_state
    secs = []
    tmp = tempfile.mkdtemp(prefix="nsp_ref_")
    for k in range(args.warmup + args.steps):
        m = k % MEMBERS
        d = os.path.join(tmp, "m%d" % m)
        if not os.path.isdir(d):
            write_state(member_fields(m), d)
        rd = build_ref.run("c0", "time", d, steps_per_sample, nsteps_build=steps_per_sample)
        txt = open(os.path.join(rd, "stdout.txt")).read()
        rec = json.loads(txt.split("REFTIME", 1)[1].strip().splitlines()[0])
        if k >= args.warmup:
            secs.append(rec["seconds"])
    value = args.steps * steps_per_sample / sum(secs)
    line.update({
        "value": value, "ms_per_step": 1e3 * sum(secs) / (args.steps * steps_per_sample),
        "ns_per_step_dof": 1e9 * sum(secs) / (args.steps * steps_per_sample) / DOF,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded perturbations)",
        "config": {"workload": WORKLOAD, "members": MEMBERS, "precision": "fp64",
                   "reference": "nsPipe-CUDA Main_Code built with nvcc -O3 sm_103a, one pipe per process; each "
                                "sample = integrate() over %d steps of one member, wall clock around integrate()"
                                % steps_per_sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "reference",
                         "sample": "%d samples x %d steps of single members on the GPU (the reference has no CPU "
                                   "implementation of the step)" % (args.steps, steps_per_sample)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    })
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ uneven batch (supplementary line)
UNEVEN = [  # (members, NR, NT, NZ, Re low, Re high): 32x64, 48x128, 96x192 modes
    (16, 48, 32, 65, 2000.0, 2400.0),
    (8, 64, 48, 129, 2400.0, 3000.0),
    (4, 96, 96, 193, 3000.0, 4000.0),
]
UNEVEN_DT, UNEVEN_AMP = 0.006, 0.05  # dt = 0.003 R/U_b


UNEVEN_WORKLOAD = ("uneven batch: 16 pipes NR=48 x 32 x 64 modes (Re 2000-2400), 8 NR=64 x 48 x 128 (Re 2400-3000), "
                   "4 NR=96 x 96 x 192 (Re 3000-4000); dt=0.003R/U_b, L=4piR, amplitude 0.05")


def measure_uneven(args, device=0, barrier=None, max_over_ranks=None):
    """Mixed-precision uneven batch: 28 pipes of three resolutions with Re spread
    within each; member-steps/s and ns/(step.dof) over the whole batch, the plain
    FP64 form on the same batch, and the execution choices (one group per shape,
    one operator set per Re, groups as parallel graph branches).  Returns a dict."""
    import torch
    import nspipe_gb300 as nsp
    barrier = barrier or torch.cuda.synchronize
    max_over_ranks = max_over_ranks or (lambda x: x)
    prm, fields, dof = [], [], 0
    k = 0
    for n, nr, nt, nz, lo, hi in UNEVEN:
        for i in range(n):
            re = lo + (hi - lo) * i / max(1, n - 1)
            prm.append(nsp.make_params(nr, nt, nz, re, UNEVEN_DT, 2.0 * PI2))
            fields.append(nsp.seeded_field(nr, nt, nz, 2.0 * PI2, UNEVEN_AMP, 4000 + k))
            dof += 3 * nr * nt * nz
            k += 1

    def timed(precision):
        t_setup = time.perf_counter()
        st = nsp.Stepper(prm, precision=precision, device=device)  # 28 parameter sets, autotune, graph
        t_setup = time.perf_counter() - t_setup
        for m, f in enumerate(fields):
            st.set_state(m, f)
        desc = st.describe()
        stream = torch.cuda.Stream()
        st.set_stream(stream.cuda_stream)
        st.step(args.warmup, check=False)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(device) as clk:
            with torch.cuda.stream(stream):
                e0.record(stream)
                iters = st.step(args.steps, check=False)
                e1.record(stream)
            barrier()
        sec = max_over_ranks(e0.elapsed_time(e1) / 1e3)
        launches = st.kernel_launches()
        finite = all(d.status == 0 for d in st.diag_all())
        st.set_stream(0)
        st.close()
        desc["setup_seconds"] = round(t_setup, 3)
        return sec, iters, clk.summary(), desc, launches, finite

    sec, iters, clocks, desc, launches, finite = timed(nsp.NSP_MIXED)
    n = len(prm)
    out = {"value": n * args.steps / sec, "unit": UNIT, "ms_per_step": 1e3 * sec / args.steps,
           "ns_per_step_dof": 1e9 * sec / args.steps / dof, "iters_mean": float(iters.mean()),
           "gpu_launches": int(launches), "clocks": clocks, "all_members_finite": finite,
           "members": n, "workload": UNEVEN_WORKLOAD, "execution": desc}
    if not args.no_fp64_compare:
        sec64, it64, _, _, _, fin64 = timed(nsp.NSP_FP64)
        out["fp64_form"] = {"value": n * args.steps / sec64, "unit": UNIT, "ms_per_step": 1e3 * sec64 / args.steps,
                            "iters_mean": float(it64.mean()), "mixed_over_fp64": sec64 / sec,
                            "all_members_finite": fin64}
    return out


def run_uneven(args):
    """The uneven batch as its own JSON line (--workload uneven)."""
    import torch
    torch.cuda.set_device(0)
    u = measure_uneven(args)
    out = {"metric": METRIC, "value": u["value"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": u["ms_per_step"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64+f32",
           "data": "synthetic: seeded divergence-free perturbations of Hagen-Poiseuille flow",
           "config": {"workload": UNEVEN_WORKLOAD, "members_per_gpu": u["members"], "precision": "mixed",
                      "execution": u["execution"]},
           "ns_per_step_dof": u["ns_per_step_dof"], "iters_mean": u["iters_mean"], "gpu_launches": u["gpu_launches"],
           "clocks": u["clocks"], "all_members_finite": u["all_members_finite"]}
    if "fp64_form" in u:
        out["fp64_form"] = u["fp64_form"]
    print(json.dumps(out))
    return 0


# ------------------------------------------------------------------ our arm
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--members", type=int, default=MEMBERS)
    ap.add_argument("--no-fp64-compare", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="ensemble", choices=["ensemble", "uneven"],
                    help="ensemble: the headline 64-member workload; uneven: the mixed three-resolution batch")
    ap.add_argument("--split", action="store_true",
                    help="strong scaling: shard one ensemble of --members pipes across the ranks "
                         "(default: every rank advances its own --members pipes, weak scaling)")
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven-batch sub-measurement")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "uneven":
        return run_uneven(args)

    import numpy as np
    import torch
    import nspipe_gb300 as nsp

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if not dist:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    prec = nsp.NSP_MIXED if args.precision == "mixed" else nsp.NSP_FP64
    if args.split:  # one fixed ensemble, partitioned: this rank owns members [lo, hi)
        from nspipe_gb300.ensemble import shard
        lo, hi = shard(args.members, world, rank)
        total_members = args.members
    else:  # every rank its own ensemble of --members pipes
        lo, hi = rank * args.members, (rank + 1) * args.members
        total_members = args.members * world
    M = hi - lo
    fields = [member_fields(m) for m in range(lo, hi)]

    def make(precision):
        st = nsp.Stepper([nsp.make_params(NR, NT, NZ, RE, DT, LZ) for _ in range(M)], precision=precision, device=local)
        for m in range(M):
            st.set_state(m, fields[m])
        return st

    def device_timed(st, K, W):
        stream = torch.cuda.Stream()
        st.set_stream(stream.cuda_stream)
        st.step(W)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            with torch.cuda.stream(stream):
                e0.record(stream)
                iters = st.step(K)
                e1.record(stream)
            barrier()
        ms = e0.elapsed_time(e1)
        st.set_stream(0)
        return ms / 1e3, iters, clk.summary()

    t_setup = time.perf_counter()
    st = make(prec)
    t_setup = time.perf_counter() - t_setup
    describe = st.describe()  # graph, autotuned linear-pass block, theta-transform path
    describe["setup_seconds"] = round(t_setup, 3)
    sec, iters, clocks = device_timed(st, args.steps, args.warmup)
    launches = st.kernel_launches()
    sec_max = max_over_ranks(sec)
    total_member_steps = total_members * args.steps
    value = total_member_steps / sec_max

    # Roofline of the dominant kernel: CUDA-event timing of standalone launches.
    stage_ms = st.profile_stages(reps=5)
    names = ["nl_theta_inv", "nl_z", "nl_theta_fwd", "linear_k", "converge_k"]
    csz = 8 if prec == nsp.NSP_MIXED else 16
    NTP, NZR = 3 * NT // 2, 3 * (NZ - 1)
    alg_bytes = [  # algorithmic bytes per launch (all members)
        M * (3 * S * 16 + 9 * NR * NTP * NZ * csz),           # read u (stencil counted once), write G
        M * (9 * NR * NTP * NZ * csz + 3 * NR * NTP * (NZ - 1) * csz),  # read G, write H
        M * (3 * NR * NTP * (NZ - 1) * csz + 3 * S * csz),    # read H, write N (mixed: FP32)
        # predictor pass (the one timed), bytes per point: FP64 form, read u^n, N, V, write
        # u_1 and RHSW (5 x 3 x 16); mixed, read u^n (3 x 16), N and u^n's FP32 mirror (6 x 8),
        # write u_1 (3 x 16), RHSW, the new FP32 mirror and its d_r (9 x 8) -- the per-set
        # tables (factors, V, stencils) are shared by the members and L2-resident
        M * S * (6 * 16 + 15 * 8 if prec == nsp.NSP_MIXED else 15 * 16),
        M * 64,
    ]
    dom = int(np.argmax(stage_ms[:4]))
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes[dom] / (stage_ms[dom] * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("%s_%s" % (names[dom], args.precision))
        except ValueError:
            traffic = None
    roofline = {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
                "algorithmic_bytes_per_launch": alg_bytes[dom], "launch_ms": stage_ms[dom],
                "stage_ms": dict(zip(names, [float(x) for x in stage_ms]))}
    # The linear pass.  FP64 form: bound by the FP64 pipe (FP64 ~1/64 of FP32 on GB300);
    # FP64 flops per grid point of the predictor: explicit Laplacian 84, coefficients 7,
    # right-hand sides 20 + 12, step-invariant part 12, divergence 37, pressure solve 26,
    # gradient and +/- 41, three Helmholtz solves 78, influence correction and r/theta 30:
    # 347; corrector 242 (right-hand side 12, divergence 37, pressure solve 26, gradient
    # and +/- 41, Helmholtz solves 78, correction 30, convergence measure 18).  Mixed form:
    # its stencils, solves and corrections run in FP32 and double-float, leaving 12 FP64
    # flops per point in each pass (the split of u^n and the stored state; the increment
    # pass's update of u) -- the pass is latency-bound, not FP64-bound.
    if names[dom] == "linear_k":
        fp64_peak = st.fp64_peak_tflops()
        mixed = prec == nsp.NSP_MIXED
        fl = (12.0 if mixed else 347.0) * S * M
        ach = fl / (stage_ms[dom] * 1e-3) / 1e12
        roofline["compute_bound"] = "latency (barrier and memory-latency stalls)" if mixed else "fp64"
        roofline["fp64"] = {"achieved_tflops": ach, "peak_tflops": fp64_peak, "frac": ach / fp64_peak,
                            "algorithmic_flops_per_launch": fl, "peak_source": "measured live (nsp_measure_fp64_peak)"}
        # The corrector pass, bytes per point: FP64 form, read N, RHSW, V, u_i, write u_{i+1}
        # (15 x 16); mixed (the increment pass), read u_i (3 x 16), N, RHSW and u_i's FP32
        # mirror (9 x 8), write u_{i+1} (3 x 16), RHSW, the FP32 mirror and its d_r (9 x 8).
        lin = st.profile_linear(5)
        fl_c = (12.0 if mixed else 242.0) * S * M
        by_c = M * S * ((6 * 16 + 18 * 8) if mixed else 15 * 16)
        roofline["corrector"] = {"launch_ms": float(lin[1]), "fp64_frac": fl_c / (lin[1] * 1e-3) / 1e12 / fp64_peak,
                                 "hbm_frac": by_c / (lin[1] * 1e-3) / 1e9 / peak,
                                 "algorithmic_flops_per_launch": fl_c, "algorithmic_bytes_per_launch": by_c}

    # End to end through the C ABI with host buffers: every step is one nsp_step_host
    # call -- H2D of all members' state from pinned memory, one step, D2H of all
    # members' state into pinned memory (the members in chunks, so that the copies of
    # one chunk overlap the compute of the others).  Wall clock, max over ranks.
    def pinned(n):
        return torch.zeros(n, dtype=torch.complex128).pin_memory().numpy()

    def e2e_timed(stp):
        host_in, host_out = pinned(3 * M * S), pinned(3 * M * S)  # member-major: u_r, u_t, u_z per member
        host_in[:] = stp.pack(fields)
        for _ in range(args.warmup):
            stp.step_host(1, host_in, out=host_out)
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            stp.step_host(1, host_in, out=host_out)
            host_in, host_out = host_out, host_in
        barrier()
        e2e_sec = max_over_ranks(time.perf_counter() - t0)
        return {"value": total_member_steps / e2e_sec, "unit": UNIT, "h2d_bytes_per_step": M * 3 * S * 16,
                "d2h_bytes_per_step": M * 3 * S * 16}

    e2e = e2e_timed(st)

    # Plain FP64 form on the same ensemble (the metric's comparison; the drop-in form),
    # device-timed and end to end.
    fp64 = None
    if prec == nsp.NSP_MIXED and not args.no_fp64_compare:
        st64 = make(nsp.NSP_FP64)
        sec64, it64, _ = device_timed(st64, args.steps, args.warmup)
        sec64 = max_over_ranks(sec64)
        v64 = total_member_steps / sec64
        fp64 = {"value": v64, "unit": UNIT, "ms_per_step": 1e3 * sec64 / args.steps,
                "ns_per_step_dof": 1e9 * sec64 / args.steps / (total_members * DOF),
                "iters_mean": float(it64.mean()), "mixed_over_fp64": value / v64, "e2e": e2e_timed(st64)}
        st64.close()

    # The uneven mixed batch (three resolutions, Re spread), every rank its own batch.
    uneven = None
    if not args.no_uneven:
        uneven = measure_uneven(args, device=local, barrier=barrier, max_over_ranks=max_over_ranks)
        if world > 1:
            uneven["value"] *= world
            if "fp64_form" in uneven:
                uneven["fp64_form"]["value"] *= world

    out = None
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sec_max / args.steps, "higher_is_better": True,
            "scaling": "strong" if args.split else "weak", "vs_baseline": None,
            "dtype": "f64+f32" if prec == nsp.NSP_MIXED else "f64",
            "data": "synthetic: seeded divergence-free perturbations of Hagen-Poiseuille flow",
            "config": {"workload": WORKLOAD, "members_per_gpu": M, "precision": args.precision,
                       "parallelism": ("one ensemble of %d pipes sharded across %d GPUs" % (total_members, world)
                                       if args.split else "every GPU its own ensemble (dp%d)" % world)
                                      + ", no collective",
                       "l2": "inputs larger than L2: %.2f GB of member state per GPU" % (M * 9 * S * 16 / 1e9),
                       "execution": describe},
            "ns_per_step_dof": 1e9 * sec_max / args.steps / (total_members * DOF),
            "iters_mean": float(iters.mean()),
            "gpu_launches": int(launches),
            "clocks": clocks,
            "roofline": roofline,
            "fp64_form": fp64,
            "e2e": e2e,
            "uneven": uneven,
        }
        if world == 1 and not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline()
        print(json.dumps(out))
    st.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
