#!/usr/bin/env python3
"""Steps/s of the channel-flow time step on GB300.

Workload: turbulent channel at Re_tau = 180, grid 128 x 129 x 128
(nnx = 128 streamwise, nnz = 128 -> 129 wall-normal Chebyshev points,
nny = 128 spanwise), box 4 pi x 2 x 4 pi / 3, dt = 2e-4 (the reference's own
time step), started from the laminar profile plus a seeded divergence-free
perturbation.  One "step" is one iteration of the
reference main loop: getnonlinear followed by the per-mode and (0,0)-mode
solves.  Synthetic, seeded initial data; no dataset is involved.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64]
    python bench.py --impl reference     # the reference algorithm on the host CPU

Under torchrun (N > 1) every rank advances its own independent channel
(replicas; the reference's decomposition of one channel needs an all-to-all
per transform, so one channel stays on one GPU); value = all steps / max time.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)



def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--precision", choices=["fp64", "mixed", "mixed_fp64solve"], default="mixed")
    p.add_argument("--config", default="c3_retau180_128")
    p.add_argument("--grid", default=None,
                   help="nnx,nny,nnz in place of the config's grid (same box, Reynolds number and time "
                        "step): smaller cases of a workload's kernels, for profiling")
    p.add_argument("--zpad", default="auto",
                   help="product-grid intervals in z: 0 = 2*nnz (reference), 'auto' = smallest "
                        "exact 2,3,5-smooth grid (2*zpad > 3*nnz)")
    p.add_argument("--e2e-steps", type=int, default=20)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--ensemble", type=int, default=96,
                   help="channels of the batched-ensemble measurement (0: skip)")
    p.add_argument("--accuracy-steps", type=int, default=None,
                   help="mixed path: steps of the accuracy comparison against the FP64 path (0: skip; "
                        "default 1000 for the Re_tau 180 channel, 200 for the Re_tau 550 channel)")
    p.add_argument("--no-autotune", action="store_true",
                   help="keep the launch rules instead of the autotuner's measured choice")
    return p.parse_args()


def resolve_zpad(z, nnz):
    if z != "auto":
        return int(z)
    m = 3 * nnz // 2 + 1
    while True:
        n = 2 * m
        for p in (2, 3, 5):
            while n % p == 0:
                n //= p
        if n == 1:
            return m
        m += 1


def max_over_ranks(x, dist, device):
    """The largest x over the ranks (x itself without a process group): the
    time of the slowest replica sets the job's time."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world, steps, seconds):
    """Whole-job steps/s of `world` independent replicas that each took
    `steps` steps in at most `seconds` (weak scaling: every rank advances its
    own channel)."""
    return world * steps / seconds


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# the arithmetic of each precision of the library
DTYPES = {
    "fp64": "f64",
    "mixed": "f64 state; f32 x/y FFTs and products; exact fixed-point tcgen05 z transforms (bf16 digits, exact "
             "f32 level sums); f64 curl and recurrences; solve as f64 update c + delta with delta from "
             "compensated f32 (about 2^-38), A^-1 r in f32; (0,0) mode f64",
    "mixed_fp64solve": "f64 state; f32 x/y FFTs and products; exact fixed-point tcgen05 z transforms (bf16 "
                       "digits, exact f32 level sums); f64 curl; f64 tau solve for every mode",
}


def workload_config(args):
    from channel_flow_gb300 import config
    cfg = config.CONFIGS[args.config]
    if args.grid:
        nx, ny, nz = (int(v) for v in args.grid.split(","))
        cfg = config.ChannelConfig(nx, ny, nz, cfg.aphi, cfg.beta, cfg.dt, cfg.re, cfg.re_p)
    return cfg


def start_state(cfg, seed):
    """The seeded start of a workload: the laminar profile plus a 10%
    divergence-free perturbation, or for the Re_tau 550 channel the wall-law
    (log-law) mean profile plus the 10% perturbation."""
    from channel_flow_gb300 import fields
    return fields.turbulent_start_state(cfg, seed=seed, loglaw=cfg.re >= 500.0)


def workload_name(cfg):
    """The physical workload alone (grid, box, time step, Reynolds number):
    both arms print the same string; the arithmetic (precision) and the
    wall-normal product grid are separate config keys."""
    return (f"channel {cfg.nnx}x{cfg.nnz + 1}x{cfg.nny} (nnx x wall-normal x nny), "
            f"box {2 * cfg.aphi:g}pi x 2 x {2 * cfg.beta:.4g}pi, dt={cfg.dt:g}, re={cfg.re:g}, "
            f"re_p={cfg.re_p:g}, seeded {'log-law' if cfg.re >= 500.0 else 'laminar'} mean + 10% "
            f"divergence-free perturbation")


# --------------------------------------------------------------------------
# algorithmic work per kernel launch (bytes read + written once, FP64 flops)
# --------------------------------------------------------------------------
def kernel_work(cfg, zpad=0, precision="fp64", recover_df=False):
    N = cfg.nnz
    NZ = N + 1
    KX, KY = cfg.nnx // 2, cfg.nny
    PX, PY = 3 * cfg.nnx // 2, 3 * cfg.nny // 2
    MZ = zpad or 2 * N
    MP = MZ + 1
    modes = KX * KY
    c = 16  # complex FP64

    def fft_flops(n):
        return 5.0 * n * math.log2(n)

    w = {}
    w["k_zc2v"] = (6 * NZ * modes * c + 6 * MP * modes * c, 6 * modes * fft_flops(2 * MZ))
    w["k_yinv"] = (6 * MP * modes * c + 6 * MP * PY * KX * c, 6 * MP * KX * fft_flops(PY))
    w["k_xprod"] = (6 * MP * PY * KX * c + 3 * MP * PY * KX * c,
                    MP * PY * (5 * fft_flops(PX) + 9 * PX))
    w["k_yfwd"] = (3 * MP * PY * KX * c + 3 * MP * modes * c, 3 * MP * KX * fft_flops(PY))
    w["k_zcurl"] = (3 * MP * modes * c + 4 * NZ * modes * c,
                    modes * (3 * fft_flops(2 * MZ) + 2 * fft_flops(2 * N)))
    ne, no = N // 2 + 1, N // 2
    stride = 2 * (ne * ne + no * no)
    # distinct k^2 values decide the matrix bytes
    import numpy as np
    from channel_flow_gb300.fields import wavenumbers
    ia, ib = wavenumbers(cfg)
    k2 = (ia[None, :] ** 2 + ib[:, None] ** 2)
    k2[KY // 2, :] = 0.0
    nk2 = len(np.unique(k2[k2 != 0.0]))
    nsolve = int((k2 != 0.0).sum())
    w["k_solve"] = ((nk2 + 1) * stride * 8 + 12 * NZ * modes * c,
                    nsolve * (8 * (ne * ne + no * no) + 2 * fft_flops(2 * N)))
    if precision == "fp64":
        return w
    # mixed path: FP32 x/y work halves the bytes; the z transforms are exact
    # GEMMs on bf16 digit planes (B images in, FP32/FP64 out: 3 planes for Z1,
    # 4 for Z2 and GL); the solve reads A^-1 (B - A) as (hi, lo) floats and
    # A^-1 as floats per k^2 group
    for k in ("k_yinv", "k_xprod", "k_yfwd"):
        w[k] = (w[k][0] // 2, w[k][1])
    cols = 2 * modes

    def kp(k):
        return (k + 15) // 16 * 16

    img = 4 * 2  # four bf16 planes per element (Z2, GL: 10 digit products)
    # Z1: three planes of 8-bit digits, 6 products, where K (padded) <= 204
    np1 = 3 if kp(NZ) <= 204 else 4
    img1, prod1 = np1 * 2, (6 if np1 == 3 else 10)
    w["k_tc_split_z1"] = (6 * NZ * cols * 8 + 6 * kp(NZ) * cols * img1, 0)
    w["k_tc_gemm_z1"] = (6 * kp(NZ) * cols * img1 + 6 * MP * cols * 4, 6 * prod1 * 2 * 256 * cols * kp(NZ))
    w["k_tc_split_z2"] = (3 * MP * cols * 4 + 3 * kp(MP) * cols * img, 0)
    # Z2 and GL run one 128-row tile (rows 0..N-1); row N is formed beside the digits
    w["k_tc_gemm_z2"] = (3 * kp(MP) * cols * img + 3 * N * cols * 8, 3 * 10 * 2 * N * cols * kp(MP))
    # FP64 flops, an FMA counting 2 as in the DGEMM rate: per (mode, re/im,
    # row) 7 for h_v (the G product, the recurrence, k^2 H2 + D G), 3 for h_g
    w["k_curl"] = (3 * NZ * cols * 8 + 2 * kp(NZ) * cols * img, modes * NZ * 2 * 10)
    w["k_tc_gemm_gl"] = (2 * kp(NZ) * cols * img + 2 * N * cols * 8, 2 * 10 * 2 * N * cols * kp(NZ))
    w["k_inc_solve"] = (nk2 * stride * (8 + 4) + 8 * NZ * modes * c,
                        nsolve * 2 * (2 * (ne * ne + no * no)) * 2)
    # FP64 flops per (mode, re/im, row): 3 recurrence FMAs and the four
    # outputs (16) in the FP64 form; the double-float form leaves one FP64
    # addition per output
    w["k_inc_recover"] = (6 * NZ * modes * c, nsolve * NZ * 2 * (4 if recover_df else 22))
    return w


# which pipe bounds each kernel's counted flops: the exact GEMMs' digit
# products run on the bf16 tensor pipe; the curl recurrences, the recovery and
# every kernel of the FP64 path count FP64 operations; the mixed path's FP32
# FFT and product kernels are bound by HBM alone
TENSOR_KERNELS = ("k_tc_gemm_z1", "k_tc_gemm_z2", "k_tc_gemm_gl")
FP64_MIXED_KERNELS = ("k_curl", "k_inc_recover", "k_solve")


def step_roofline(work, precision, ms_per_step, hbm_gbs, tensor_tflops, fp64_tflops):
    """Whole-step roofline: T_roof = sum over the step's kernels of
    max(bytes_k / BW_HBM, flops_k / peak_k), peak_k being the bf16 tensor rate
    for the exact GEMMs and the FP64 rate for FP64 work; achieved =
    T_roof / T_measured (1.0 = every kernel at its own bound, run back to
    back).  `work` maps kernel -> (bytes, flops) per step."""
    per = {}
    total = 0.0
    for k, (nb, nf) in work.items():
        t_mem = nb / (hbm_gbs * 1e9)
        if k in TENSOR_KERNELS:
            t_fl, pipe = nf / (tensor_tflops * 1e12), "tensor"
        elif precision == "fp64" or k in FP64_MIXED_KERNELS:
            t_fl, pipe = nf / (fp64_tflops * 1e12), "fp64"
        else:
            t_fl, pipe = 0.0, "none"
        t = max(t_mem, t_fl)
        total += t
        per[k] = {"roof_us": t * 1e6, "bound": "hbm" if t_mem >= t_fl else pipe}
    return {"t_roof_ms": total * 1e3, "t_measured_ms": ms_per_step,
            "achieved": total * 1e3 / ms_per_step, "kernels": per}


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.idx = device_index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        if sm:
            out = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


# --------------------------------------------------------------------------
# CPU baseline / reference arm: the reference algorithm restated on the host
# --------------------------------------------------------------------------
def cpu_reference_rate(cfg, seconds, warmup=1, steps=None):
    import oracle
    from channel_flow_gb300 import fields
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    o = oracle.Oracle.from_config(cfg)
    o.setup()
    o.set_state(start_state(cfg, seed=0))
    o.getnonlinear()
    o.solve()
    for _ in range(warmup):
        o.step(1)
    if steps is None:
        t = time.perf_counter()
        o.step(1)
        one = time.perf_counter() - t
        steps = max(1, int(seconds / max(one, 1e-6)))
    t = time.perf_counter()
    o.step(steps)
    el = time.perf_counter() - t
    return steps / el, threads, steps, el


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from channel_flow_gb300 import config
    cfg = workload_config(args)
    rate, threads, steps, el = cpu_reference_rate(cfg, 0, warmup=args.warmup, steps=args.steps)
    sample = (f"{steps} full time steps of the {cfg.nnx}x{cfg.nnz + 1}x{cfg.nny} workload "
              f"(CPU restatement of the reference algorithm, 12+6 padded transforms, explicit inverses)")
    line = {
        "impl": "reference", "metric": "steps/s", "value": rate, "unit": "steps/s",
        "n_gpus": world, "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 / rate,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded laminar profile + 10% divergence-free perturbation)",
        "config": {"workload": workload_name(cfg), "grid_points": cfg.points, "precision": "fp64",
                   "zpad": 2 * cfg.nnz, "parallelism": "host threads (rank 0 only)"},
        "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    rank, world, local = dist_env()
    import numpy as np
    import torch
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from channel_flow_gb300 import Channel, build as cbuild, config, fields
    if rank == 0:
        cbuild.build()
    if dist:
        dist.barrier()
    cfg = workload_config(args)
    args.zpad = resolve_zpad(args.zpad, cfg.nnz)
    if args.accuracy_steps is None:
        args.accuracy_steps = 200 if args.config.startswith("c4") else 1000
    st = start_state(cfg, seed=rank)
    ch = Channel(cfg, precision=args.precision, zpad=args.zpad, device=local)
    stream = torch.cuda.Stream(device=local)
    ch.set_stream(stream.cuda_stream)
    ch.upload_state(st)
    ch.getnonlinear()
    ch.solve()
    # launch shapes and FFT radix orders by measurement (chf_autotune; cached
    # for the later handles of this grid in the process)
    tuning = ch.tuning() if args.no_autotune else ch.autotune(3)
    ch.step(max(3, args.warmup))
    ch.synchronize()
    # ---- timed region (device events on the library's stream)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    nvtx_push("chf_timed_steps")  # lets an ncu launch list select the timed steps
    e0.record(stream)
    ch.step(args.steps)  # pairs of steps replay the library's captured graph
    e1.record(stream)
    torch.cuda.synchronize()
    nvtx_pop()
    if dist:
        dist.barrier()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    # ---- per-kernel breakdown: a separate pass with an event pair around
    # every launch (direct launches; not part of the timed region above)
    nprof = max(2, min(args.steps, 20))
    ch.profile(True)
    ch.profile_reset()
    ch.step(nprof)
    ch.synchronize()
    prof = ch.profile_report()
    ch.profile(False)
    prof_ms = sum(v[1] for v in prof.values()) / nprof
    diag = ch.diagnostics()
    t_max = max_over_ranks(ms, dist, f"cuda:{local}")
    value = replica_rate(world, args.steps, t_max / 1e3)
    # ---- end to end through the C ABI with pinned host buffers: every step
    # uploads the module arrays, advances one step and downloads them
    host = {}
    for k, a in st.items():
        host[k] = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
        host[k][...] = a
    ch.set_stream(None)
    ch.upload_state(host)
    ch.getnonlinear()
    ch.solve()
    h2d = sum(a.nbytes for a in host.values())
    ne2e = max(1, args.e2e_steps)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(ne2e):
        out = ch.step_host(host, 1)
    el = time.perf_counter() - t0
    e2e_t = max_over_ranks(el, dist, f"cuda:{local}")
    e2e = {"value": replica_rate(world, ne2e, e2e_t), "unit": "steps/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": sum(a.nbytes for a in out.values()),
           "what": "chf_step_host(1) on pinned host module arrays: all 14 arrays up and down every step, "
                   "copies overlapped with the step"}
    kernels_per_step = ch.kernels_per_step()
    ch.close()
    # FP64 path on the same start: its steps/s (device events) and, for the
    # mixed form, the velocity error after --accuracy-steps steps of both paths
    accuracy = None
    fp64_rate = None
    other_rates = {}
    if args.precision != "fp64":
        def device_rate(prec, k):
            ref = Channel(cfg, precision=prec, zpad=args.zpad, device=local)
            rs = torch.cuda.Stream(device=local)
            ref.set_stream(rs.cuda_stream)
            ref.upload_state(st)
            ref.getnonlinear()
            ref.solve()
            ref.step(max(3, args.warmup))
            ref.synchronize()
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            f0.record(rs)
            ref.step(k)
            f1.record(rs)
            torch.cuda.synchronize()
            ref.close()
            return k / (f0.elapsed_time(f1) / 1e3)

        fp64_rate = device_rate("fp64", max(2, min(args.steps, 30)))
        # the other mixed form beside the headline one
        for prec in ("mixed", "mixed_fp64solve"):
            if prec != args.precision:
                other_rates[prec] = device_rate(prec, max(2, min(args.steps, 100)))
        if args.accuracy_steps > 0:
            accuracy = accuracy_vs_fp64(Channel, cfg, st, args.zpad, local, args.accuracy_steps,
                                        forms=("mixed", "mixed_fp64solve"))
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    # ---- roofline of the dominant kernel
    work = kernel_work(cfg, args.zpad, args.precision, recover_df="double-float recovery" in tuning)
    kname = max((k for k in prof if prof[k][0] > 0), key=lambda k: prof[k][1])
    launches, kms = prof[kname]
    avg_ms = kms / launches
    nbytes, nflops = work.get(kname, (0, 0))
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved_gbs = nbytes / (avg_ms / 1e3) / 1e9
    traffic = read_traffic(kname + ("_f32" if args.precision != "fp64" and kname in ("k_yinv", "k_xprod", "k_yfwd") else ""),
                           f"{cfg.nnx}x{cfg.nnz + 1}x{cfg.nny}")
    roofline = {"bound": "hbm", "kernel": kname, "achieved": achieved_gbs, "peak": hbm_peak,
                "unit": "GB/s", "frac": achieved_gbs / hbm_peak,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if "hbm_gbs" in peaks else "fallback",
                "traffic": traffic, "algorithmic_bytes": nbytes, "avg_launch_ms": avg_ms}
    fp64_peak = fp64_peak_tflops(torch, f"cuda:{local}")
    # the step's kernels that ran in the timed graph (the (0,0) mode solve runs
    # beside k_inc_solve and moves no operator bytes)
    ran = {k: v for k, v in work.items() if prof.get(k, (0, 0))[0] > 0}
    roofline["step"] = step_roofline(ran, args.precision, t_max / args.steps, hbm_peak,
                                     peaks.get("bf16_tflops_sustained", 1700.0), fp64_peak)
    roofline["step"]["peaks"] = ("HBM: MEASURED_PEAKS.json hbm_gbs; tensor: bf16_tflops_sustained "
                                 "(measured); FP64: cuBLAS DGEMM 4096^3 measured in this run")
    if args.precision == "fp64":
        # the FP64 path's kernels are bound by the FP64 pipe: their rate against
        # the measured DGEMM peak
        roofline.update({"fp64_tflops_achieved": nflops / (avg_ms / 1e3) / 1e12,
                         "fp64_tflops_peak": fp64_peak,
                         "fp64_peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                         "fp64_frac": nflops / (avg_ms / 1e3) / 1e12 / fp64_peak})
    else:
        roofline.update({"arith_tflops": nflops / (avg_ms / 1e3) / 1e12,
                         "arith_note": "the kernel's algorithmic flops per second, computed in FP32 "
                                       "(packed f32x2, compensated): not an FP64 rate"})
    kernels = {k: {"launches": v[0], "ms_total": v[1], "share": v[1] / max(1e-9, sum(x[1] for x in prof.values()))}
               for k, v in prof.items() if v[0] > 0}
    line = {
        "metric": "steps/s", "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPES[args.precision],
        "data": "synthetic (seeded laminar profile + 10% divergence-free perturbation)",
        "config": {"workload": workload_name(cfg),
                   "grid_points": cfg.points, "precision": args.precision, "zpad": args.zpad,
                   "parallelism": f"replicas x{world}", "tuning": tuning,
                   "l2": "inputs larger than L2: >0.9 GB touched per step vs 129 MB L2"},
        "grid_point_steps_per_s": value * cfg.points,
        "gpu_launches": kernels_per_step * args.steps,
        "profile_pass": {"steps": nprof, "ms_per_step_sum_of_kernels": prof_ms,
                         "note": "per-kernel event pairs, direct launches; the headline is timed without them"},
        "clocks": clk,
        "e2e": e2e,
        "roofline": roofline,
        "kernels": kernels,
        "energy_after": diag["energy"],
    }
    if accuracy is not None:
        line["accuracy"] = accuracy
    if args.ensemble > 0:
        line["ensemble"] = ensemble_rate(args.ensemble, local)
    if fp64_rate is not None:
        line["fp64_steps_per_s"] = fp64_rate
        line["mixed_over_fp64"] = value / world / fp64_rate
        for prec, r in other_rates.items():
            line[prec] = {"steps_per_s": r, "over_fp64": r / fp64_rate, "dtype": DTYPES[prec],
                          "timing": "device events, the same start, chf_step graph replays"}
    if world == 1 and not args.no_cpu_baseline:
        rate, threads, steps, el = cpu_reference_rate(cfg, args.cpu_seconds)
        line["cpu_baseline"] = {
            "value": rate, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": f"{steps} full time steps ({el:.1f} s) of the same workload, CPU restatement "
                      f"of the reference algorithm (oracle/), OpenMP over {threads} host threads"}
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def fp64_peak_tflops(torch, device):
    """FP64 throughput of this GPU, measured now: best of three cuBLAS DGEMMs
    of size 4096 (2 n^3 flops each)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=device)
    b = torch.randn(n, n, dtype=torch.float64, device=device)
    torch.matmul(a, b)
    torch.cuda.synchronize(device)
    best = 0.0
    for _ in range(3):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize(device)
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12)
    return best


def ensemble_configs(n, seed=5):
    """n channels of the ensemble workload: nnz in {32, 64, 96} (33, 65, 97
    wall-normal points), nnx = nny in {32, 64}, Re_tau uniform in [100, 300],
    box 2 pi x 2 x pi, dt 2e-4 (seeded)."""
    import numpy as np
    from channel_flow_gb300 import config
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nz = (32, 64, 96)[i % 3]
        nx = (32, 64)[(i // 3) % 2]
        out.append(config.small(nnx=nx, nny=nx, nnz=nz, aphi=1.0, beta=0.5, dt=2e-4,
                                re=float(rng.uniform(100.0, 300.0)), re_p=1.0))
    return out


def ensemble_rate(n, device, forms=("mixed_fp64solve", "mixed"), steps=20, warmup=4):
    """Channel-steps/s of n uneven channels advanced by one chf_batch (channels
    of one grid stacked into one set of buffers, one graph launch per pair of
    steps), of the same channels stepped one after another on one stream
    (chf_step each, same precision), for each mixed form; and of the plain
    FP64 path one channel after another.  Host wall clock around the calls and
    a synchronize."""
    import torch
    from channel_flow_gb300 import Batch, Channel, fields
    cfgs = ensemble_configs(n)
    starts = [fields.turbulent_start_state(c, seed=100 + i) for i, c in enumerate(cfgs)]
    zpads = [resolve_zpad("auto", c.nnz) for c in cfgs]
    points = sum(c.points for c in cfgs)
    s = torch.cuda.Stream(device=device)
    # the plain FP64 path, one channel after another
    f64 = []
    for c, st, z in zip(cfgs, starts, zpads):
        ch = Channel(c, precision="fp64", zpad=z, device=device)
        ch.set_stream(s.cuda_stream)
        ch.upload_state(st)
        ch.getnonlinear()
        ch.solve()
        ch.step(2)
        f64.append(ch)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    for ch in f64:
        ch.step(steps)
    torch.cuda.synchronize(device)
    t_f64 = time.perf_counter() - t0
    for ch in f64:
        ch.close()
    out = {"channels": n, "steps": steps,
           "workload": "nnz in {32,64,96}, nnx = nny in {32,64}, Re_tau U[100,300], 2pi x 2 x pi, dt 2e-4",
           "fp64_sequential_grid_point_steps_per_s": points * steps / t_f64,
           "timing": "host wall clock around chf_batch_step + synchronize (the batch call gathers the channels "
                     "into their classes and scatters them back once per call)", "forms": {}}
    for precision in forms:
        t0 = time.perf_counter()
        b = Batch(cfgs, precision=precision, zpad=zpads, device=device)
        t_create = time.perf_counter() - t0
        for ch, st in zip(b, starts):
            ch.upload_state(st)
            ch.getnonlinear()
            ch.solve()
        b.step(warmup)
        b.synchronize()
        t0 = time.perf_counter()
        b.step(steps)
        b.synchronize()
        t_batch = time.perf_counter() - t0
        # the same channels one after another on one stream
        for ch in b:
            ch.set_stream(s.cuda_stream)
        for ch in b:
            ch.step(2)
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        for ch in b:
            ch.step(steps)
        torch.cuda.synchronize(device)
        t_seq = time.perf_counter() - t0
        for ch in b:
            ch.set_stream(None)
        finite = all(ch.diagnostics()["finite"] for ch in b)
        b.close()
        out["forms"][precision] = {
            "channel_steps_per_s": n * steps / t_batch,
            "grid_point_steps_per_s": points * steps / t_batch,
            "sequential_channel_steps_per_s": n * steps / t_seq,
            "batch_over_sequential": t_seq / t_batch,
            "batch_over_fp64_sequential": t_f64 / t_batch,
            "create_s": t_create, "finite": finite}
    return out


def accuracy_vs_fp64(Channel, cfg, st, zpad, device, nsteps, forms=("mixed",)):
    """The FP64 path and each mixed form from the same start for nsteps steps
    (after the start-up getnonlinear + solve): per form, rel-L2 of each field
    against the FP64 state, of the velocity vector (u, v, w) as a whole, of
    the pressure, and the relative differences of wall shear and energy."""
    import numpy as np
    out, extra = {}, {}
    for prec in ("fp64",) + tuple(forms):
        ch = Channel(cfg, precision=prec, zpad=zpad, device=device)
        ch.upload_state(st)
        ch.getnonlinear()
        ch.solve()
        ch.step(nsteps)
        ch.synchronize()
        out[prec] = ch.download_state()
        extra[prec] = (ch.pressure(), ch.statistics())
        ch.close()
    a = out["fp64"]
    nyq = cfg.nny // 2
    res = {}
    for prec in forms:
        b = out[prec]
        errs, num, den = {}, 0.0, 0.0
        for k in ("unp1", "vnp1", "wnp1", "omegaynp1"):
            pa = np.delete(a[k], nyq, axis=1)
            pb = np.delete(b[k], nyq, axis=1)
            d2, r2 = float(np.sum((pb - pa) ** 2)), float(np.sum(pa ** 2))
            errs[k] = (d2 / r2) ** 0.5
            if k != "omegaynp1":
                num, den = num + d2, den + r2
        vel = (num / den) ** 0.5
        pa = np.delete(extra["fp64"][0], nyq, axis=1)
        pb = np.delete(extra[prec][0], nyq, axis=1)
        errs["pressure"] = float(np.linalg.norm(pb - pa) / np.linalg.norm(pa))
        sa, sb = extra["fp64"][1], extra[prec][1]
        rel = lambda k: abs(sb[k] - sa[k]) / abs(sa[k])
        errs["wall_shear_top"] = rel("u_tau_top") * 2.0     # tau_w = u_tau^2
        errs["wall_shear_bottom"] = rel("u_tau_bottom") * 2.0
        errs["energy"] = rel("energy")
        res[prec] = {"rel_l2_vs_fp64": errs, "velocity_rel_l2": vel,
                     "velocity_component_max_rel_l2": max(errs[k] for k in ("unp1", "vnp1", "wnp1")),
                     "met": vel <= 1e-5}
    return {"steps": nsteps, "target": 1e-5, "forms": res,
            "note": "spectral coefficients without the spanwise Nyquist slot; velocity = (u, v, w) as one "
                    "vector; pressure = total head (chf_pressure); wall shear and energy from chf_statistics "
                    "(relative differences)"}


def nvtx_push(name):
    try:
        import torch
        torch.cuda.nvtx.range_push(name)
    except Exception:
        pass


def nvtx_pop():
    try:
        import torch
        torch.cuda.nvtx.range_pop()
    except Exception:
        pass


def read_traffic(kname, grid):
    """DRAM bytes per launch of kname on the grid nnx x (nnz+1) x nny from the
    committed ncu summary, if one was captured for that grid."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 3 and parts[0] == kname and parts[1] == grid:
                return float(parts[2])
    except OSError:
        pass
    return None


if __name__ == "__main__":
    sys.exit(main())
