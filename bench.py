#!/usr/bin/env python
"""Benchmark of the SpMSpV hot path (one step = one H*v product of a Krylov vector).

Workload: synthetic RHF integrals, 28 spatial / 56 spin orbitals, 14 electrons,
seed 1 (FP64, 8-fold symmetric, distributions of sfci_gb300.fcidump), Nd = 1e6.
The input vector is a power-iteration Krylov vector: v_{k+1} = top-Nd(H v_k)
(normalised) from |HF>, iterated on the device until it holds Nd determinants.
value   = merged terms/s = Nd * C / t, C = connected determinants per source
          determinant (30723 here: singles + same- and opposite-spin doubles);
e2e     = the same through the C ABI from pinned host buffers: host->device copy
          of the input, SpMSpV, device->host copy of the result, every step;
roofline= dominant kernel of the step, algorithmic bytes per launch / its mean
          launch time (CUDA events on the library's stream), against the
          measured HBM copy bandwidth.

--impl reference times the CPU implementation of the same path (the oracle
restatement of the reference algorithm, all host threads) on a bounded sample
of the same workload.  Multi-GPU (torchrun) runs independent replicas, one per
rank (weak scaling); rank 0 prints one JSON line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SpMSpV s/iter and merged terms/s at Nd=1e7; learned-screened vs plain, ΔE≤10 μEh"
UNIT = "merged terms/s"
HPSI_CAP = 60000000
# Systems of the configurations (synthetic integrals of the generator's
# distributions): 1 is the default workload; 2 has two-word keys.
SYSTEMS = {
    1: dict(M=28, ne=14, seeds=(1,), text="56 spin orbitals, 14 electrons, synthetic RHF seed 1"),
    2: dict(M=64, ne=20, seeds=(2, 3), text="128 spin orbitals, 20 electrons, synthetic UHF seeds 2 (alpha) and 3 (beta)"),
}


def connected_per_det(M, na, nb):
    va, vb = M - na, M - nb
    c2 = lambda n: n * (n - 1) // 2
    return na * va + nb * vb + c2(na) * c2(va) + c2(nb) * c2(vb) + na * va * nb * vb


def emitted_per_det(M, na, nb):
    """Raw terms the reference emits per determinant (direct and exchange separately)."""
    ne = na + nb
    va, vb = M - na, M - nb
    c2 = lambda n: n * (n - 1) // 2
    S = na * va + nb * vb
    dss = 2 * c2(na) * c2(va) if na == nb else c2(na) * c2(va) + c2(nb) * c2(vb)
    return 2 * dss + na * va * nb * vb + S * (ne + na - 1)


def workload_in(sysd=SYSTEMS[1], cache_dir=None):
    from sfci_gb300 import fcidump as fd
    d = cache_dir or os.path.join(tempfile.gettempdir(), "sfci_bench")
    os.makedirs(d, exist_ok=True)
    M, ne, seeds = sysd["M"], sysd["ne"], sysd["seeds"]
    p = os.path.join(d, "m%d_ne%d_s%s_IN" % (M, ne, "_".join(map(str, seeds))))
    if not os.path.exists(p):
        if len(seeds) == 1:
            fd.rhf_to_in_file(p + ".tmp", M, ne, seeds[0], fcidump_path=p + ".fcidump")
        else:
            fd.uhf_to_in_file(p + ".tmp", M, ne, seeds[0], seeds[1], fcidump_path=p + ".fcidump")
        os.replace(p + ".tmp", p)
    return p


def key_words(sysd):
    return 1 if 2 * sysd["M"] <= 64 else 2


def hf_key(sysd):
    hf = (1 << sysd["ne"]) - 1  # lowest ne spin orbitals, alpha/beta interleaved
    if key_words(sysd) == 1:
        return np.array([hf], np.uint64)
    return np.array([[hf & (2 ** 64 - 1), hf >> 64]], np.uint64)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms in the background."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev = dev
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# CPU baseline (oracle restatement of the reference algorithm)
# ---------------------------------------------------------------------------

def cpu_baseline(sysd, path, sample_keys, sample_amps_fn, target_s=15.0, threads=None):
    from oracle import oracle as orc
    orc.build_port()
    threads = threads or os.cpu_count() or 1
    be = orc.PortLib(words=key_words(sysd))
    be.setup(path, 2 * sysd["M"], sysd["ne"], 10 ** 7, nthread=threads)
    C = connected_per_det(sysd["M"], sysd["ne"] // 2, sysd["ne"] // 2)
    n = 100
    while True:
        k, a = sample_keys[:n], sample_amps_fn(n)
        t = time.perf_counter()
        be.spmspv(k, a, 10 ** 7, 0.0, 1.0)
        dt = time.perf_counter() - t
        if dt > target_s / 4 or n >= len(sample_keys):
            break
        n = min(len(sample_keys), int(n * min(8.0, max(2.0, target_s / max(dt, 1e-3) / 2))))
    return {"value": n * C / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "top-%d determinants of the same input vector, one SpMSpV, %.1f s" % (n, dt),
            "seconds": dt, "dets": n}


# ---------------------------------------------------------------------------

def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ["RANK"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    dist.init_process_group(backend)
    return rank, ws, local, dist


def reduce_max(dist, x, local):
    if dist is None:
        return x
    import torch
    dev = "cuda:%d" % local if torch.cuda.is_available() else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def run_reference(args, rank, ws, dist):
    if rank != 0:
        return
    from oracle import oracle as orc
    sysd = SYSTEMS[args.config]
    path = workload_in(sysd)
    threads = os.cpu_count() or 1
    orc.build_port()
    be = orc.PortLib(words=key_words(sysd))
    be.setup(path, 2 * sysd["M"], sysd["ne"], args.nd, nthread=threads)
    k1, a1, _ = be.spmspv(hf_key(sysd), np.array([1.0]), 10 ** 7, 0.0, 1.0)
    order = np.argsort(-np.abs(a1), kind="stable")
    C = connected_per_det(sysd["M"], sysd["ne"] // 2, sysd["ne"] // 2)
    # size each step for ~args.ref_step_s seconds of CPU work
    n = 200
    for _ in range(6):
        sel = np.sort(order[:n])
        t = time.perf_counter()
        be.spmspv(k1[sel], a1[sel], 10 ** 7, 0.0, 1.0)
        dt = time.perf_counter() - t
        if dt >= args.ref_step_s / 2 or n >= len(order):
            break
        n = min(len(order), int(n * min(8.0, args.ref_step_s / max(dt, 1e-3))))
    sel = np.sort(order[:n])
    ks, as_ = k1[sel], a1[sel] / np.linalg.norm(a1[sel])
    for _ in range(args.warmup):
        be.spmspv(ks, as_, 10 ** 7, 0.0, 1.0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        be.spmspv(ks, as_, 10 ** 7, 0.0, 1.0)
    dt = (time.perf_counter() - t0) / args.steps
    val = n * C / dt
    out = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "SpMSpV of a Krylov vector, " + sysd["text"],
                      "num_orb": 2 * sysd["M"], "num_e": sysd["ne"], "Nd": args.nd, "sample_dets": n,
                      "parallelism": "CPU, %d threads" % threads},
           "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": "top-%d determinants of H|HF>, one SpMSpV per step" % n},
           "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_gpu(args, rank, ws, local, dist):
    import sfci_gb300 as sg
    sg.load_library()
    sysd = SYSTEMS[args.config]
    path = workload_in(sysd)
    nd = args.nd
    M, NE, W = sysd["M"], sysd["ne"], key_words(sysd)
    ctx = sg.Context(path, 2 * M, NE, Nd=nd, hpsi_cap=HPSI_CAP, mem_budget=args.mem_budget)
    # input: v_{k+1} = top-Nd(H v_k) normalised, from |HF>, until it holds Nd dets
    hf = hf_key(sysd)
    vin = ctx.vec(nd)
    vin.upload(hf, np.array([1.0]))
    tmp = ctx.vec(HPSI_CAP)
    steps_in = 0
    while vin.len < nd and steps_in < 8:
        ctx.SpMVMtply_bucket(vin, tmp, 0.0, 1.0)
        vin.shrinkFrom(tmp)
        vin.normalize()
        steps_in += 1
    n_in = vin.len
    del tmp
    out = ctx.vec(HPSI_CAP)
    C = connected_per_det(M, NE // 2, NE // 2)
    T_conn = n_in * C
    for _ in range(args.warmup):
        ctx.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    # ---- device-resident timing
    ctx.profile(True)
    ctx.profile_reset()
    clocks = ClockSampler(local)
    clocks.start()
    barrier(dist)
    l0 = ctx.launches()
    ctx.event_record(0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        diag = ctx.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    ctx.event_record(1)
    ms = ctx.event_elapsed(0, 1) / args.steps
    wall = (time.perf_counter() - t0) / args.steps
    launches = ctx.launches() - l0
    clk = clocks.stop()
    prof = ctx.profile_read()
    ctx.profile(False)
    stats = ctx.last_stats()
    out_len = out.len
    ms_max = reduce_max(dist, ms, local)
    # ---- end to end from pinned host buffers
    keys_h, amps_h = vin.download()
    e2e_ms = None
    h2d = d2h = 0
    try:
        import torch
        pk = torch.empty(keys_h.size, dtype=torch.int64, pin_memory=True)
        pa = torch.empty(amps_h.size, dtype=torch.float64, pin_memory=True)
        pk.numpy()[:] = keys_h.reshape(-1).view(np.int64)
        pa.numpy()[:] = amps_h
        ok = torch.empty(HPSI_CAP * W, dtype=torch.int64, pin_memory=True)
        oa = torch.empty(HPSI_CAP, dtype=torch.float64, pin_memory=True)
        host = (pk.data_ptr(), pa.data_ptr(), ok.data_ptr(), oa.data_ptr())
    except Exception:
        keys_p = np.ascontiguousarray(keys_h)
        amps_p = np.ascontiguousarray(amps_h)
        ok_np = np.zeros(HPSI_CAP * W, np.uint64)
        oa_np = np.zeros(HPSI_CAP)
        host = (keys_p.ctypes.data, amps_p.ctypes.data, ok_np.ctypes.data, oa_np.ctypes.data)
    import ctypes as C_
    L = ctx.L
    vin_e = ctx.vec(nd)
    got = C_.c_uint64()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        assert L.sfci_vec_upload(vin_e.h, C_.c_void_p(host[0]), C_.c_void_p(host[1]), n_in) == 0
        d = C_.c_double()
        assert L.sfci_spmspv(ctx.h, vin_e.h, out.h, 0.0, 1.0, C_.byref(d)) == 0
        assert L.sfci_vec_download(out.h, C_.c_void_p(host[2]), C_.c_void_p(host[3]), HPSI_CAP,
                                   C_.byref(got)) == 0
    e2e_s = (time.perf_counter() - t0) / args.steps
    e2e_s = reduce_max(dist, e2e_s, local)
    tbytes = 8 * W + 8  # one determinant: key words + FP64 amplitude
    h2d = n_in * tbytes
    d2h = got.value * tbytes + 8
    if rank != 0:
        barrier(dist)
        return
    # ---- roofline of the dominant kernel
    hbm, how = peaks()
    T = stats["terms"]
    surv = stats["survivors"]
    # partition levels: generation resolves L1_BITS of the leaf hash, each level up to DIGIT_BITS more
    L1_BITS, DIGIT_BITS = 9, 9
    b = max(1, int(round(np.log2(max(stats["leaves"], 1)))))
    levels = -(-(b - min(b, L1_BITS)) // DIGIT_BITS)
    # algorithmic bytes per phase (all launches of the timed steps)
    alg = {
        "scatter": tbytes * T * args.steps,                      # generated (key, amp) terms written once
        "partition": (8.0 * W + 2 * tbytes) * T * levels * args.steps,  # per level: key (count), term in + out
        "merge": (tbytes * T + tbytes * surv) * args.steps,      # read every term once, write survivors
        "count": 0.0,                                    # keys only, kept on chip
        "select": 8.0 * surv * 6 * args.steps,
        "sort": 32.0 * out_len * 7 * args.steps,
        "other": 0.0,
    }
    kernels = {"scatter": "k_gen<SCATTER>", "partition": "k_part<COUNT,SCATTER>", "merge": "k_leafw",
               "count": "k_gen<COUNT>", "select": "select_threshold", "sort": "radix_sort_pairs", "other": "-"}
    # DRAM bytes per generated term measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum over
    # every launch of a 56-orbital Nd=1e4 run with 4 generation passes), scaled here to a launch by the
    # terms it processes
    ncu_bytes_per_term = {"scatter": 17.79, "partition": 50.53 * levels, "merge": 16.11}
    dom = max(prof, key=lambda k: prof[k][0])
    dms, dl = prof[dom]
    per_launch_bytes = alg[dom] / max(dl, 1)
    per_launch_ms = dms / max(dl, 1)
    achieved = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9 if per_launch_ms > 0 else 0.0
    traffic = (ncu_bytes_per_term[dom] * T * args.steps / max(dl, 1)) if (dom in ncu_bytes_per_term and W == 1) \
        else None  # measured for one-word keys
    value = T_conn * ws / (ms_max * 1e-3)
    e2e_val = T_conn * ws / e2e_s
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max, "s_per_iter": ms_max / 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "SpMSpV of a Krylov vector (top-Nd of H^k|HF>, k=%d), %s" % (steps_in, sysd["text"]),
                   "num_orb": 2 * M, "num_e": NE, "Nd": nd, "input_dets": n_in,
                   "connected_per_det": C, "emitted_per_det_reference": emitted_per_det(M, NE // 2, NE // 2),
                   "generated_terms_per_step": T, "merged_unique_per_step": stats["unique"],
                   "survivors_per_step": surv, "output_dets": out_len,
                   "passes": stats["passes"], "leaves": stats["leaves"], "partition_levels": levels,
                   "l2": "inputs larger than L2: %.0f GB of terms per step vs 129 MB" % (tbytes * T / 1e9),
                   "parallelism": "replicas" if ws > 1 else "1 GPU"},
        "roofline": {"bound": "hbm", "kernel": kernels[dom], "phase": dom, "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "peak_source": how, "traffic": traffic,
                     "traffic_unit": "bytes per launch", "algorithmic_bytes_per_launch": per_launch_bytes,
                     "launches": dl, "ms_per_launch": per_launch_ms},
        "phases_ms_per_step": {k: v[0] / args.steps for k, v in prof.items()},
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_s * 1e3},
        "gpu_launches": launches,
        "clocks": clk,
        "diag": diag,
    }
    if not args.no_cpu_baseline:
        keys_sorted = keys_h[np.argsort(-np.abs(amps_h), kind="stable")]
        amps_sorted = amps_h[np.argsort(-np.abs(amps_h), kind="stable")]
        res["cpu_baseline"] = cpu_baseline(sysd, path, keys_sorted,
                                           lambda n: amps_sorted[:n] / np.linalg.norm(amps_sorted[:n]),
                                           target_s=args.cpu_seconds)
    print(json.dumps(res), flush=True)
    barrier(dist)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--nd", type=int, default=1000000)
    ap.add_argument("--config", type=int, default=1, choices=sorted(SYSTEMS),
                    help="system: 1 = 56 spin orbitals / 14 electrons (the default workload), "
                         "2 = 128 spin orbitals / 20 electrons with two-word keys")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--ref-step-s", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--mem-budget", type=int, default=0,
                    help="device bytes the SpMSpV may use (0: 80%% of free); a small budget forces several "
                         "generation passes on a small case, e.g. for profiling")
    args = ap.parse_args()
    rank, ws, local, dist = dist_init()
    try:
        if args.impl == "reference":
            run_reference(args, rank, ws, dist)
        else:
            run_gpu(args, rank, ws, local, dist)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
