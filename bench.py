#!/usr/bin/env python
"""Benchmark of the SpMSpV hot path (one step = one H*v product of a Krylov vector).

Workload: synthetic RHF integrals, 28 spatial / 56 spin orbitals, 14 electrons,
seed 1 (FP64, 8-fold symmetric, distributions of sfci_gb300.fcidump), Nd = 1e6.
The input vector is a second Krylov vector built identically by both arms:
v1 = H|HF> (all 30,724 connected determinants), normalised; v2 = top-Nd of
H v1 by |amplitude| (products without the 1e-5 cut), normalised.  The GPU arm
builds it with its own product on the device, the reference arm with the CPU
restatement; the two agree to rounding (RHF spin-mirror twins that tie exactly
at the top-Nd edge may be swapped, which changes no work).
value   = merged terms/s = Nd * C / t, C = connected determinants per source
          determinant (30723 here: singles + same- and opposite-spin doubles);
e2e     = the same through the C ABI from pinned host buffers: host->device copy
          of the input, SpMSpV, device->host copy of the result, every step;
roofline= dominant kernel of the step, algorithmic bytes per launch / its mean
          launch time (CUDA events on the library's stream), against the
          measured HBM copy bandwidth; product_roofline = the whole product's
          bytes under the materialise-once model (Nd + 2 T_conn + U)(K + 8)
          over the step time;
parity  = the GPU product of the exact top-n slice that cpu_baseline times,
          against the CPU restatement's product of it (key sets, amplitudes).

--impl reference times the CPU implementation of the same path (the oracle
restatement of the reference algorithm, all host threads) on a bounded top-n
slice of the same input vector.  Multi-GPU (torchrun) runs independent
replicas, one per rank (weak scaling); rank 0 prints one JSON line.
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


INPUT_TEXT = ("third Krylov vector: v1 = H|HF>, v2 = H top_m1(v1), v3 = H top_m2(v2), input = top-Nd of v3 by "
              "|amplitude|; m1 = 2000 and m2 = 30000 scaled by 30723 / C; every vector normalised, products "
              "without the 1e-5 cut, ties kept from the highest keys")


def input_ms(sysd):
    """How many determinants of v1 and of v2 the input's later products multiply."""
    C = connected_per_det(sysd["M"], sysd["ne"] // 2, sysd["ne"] // 2)
    return max(64, 2000 * 30723 // C), max(256, 30000 * 30723 // C)


def bench_config(sysd, nd, input_dets):
    """The workload description both arms print (the reference arm adds only sample_dets)."""
    return {"workload": "SpMSpV of a Krylov vector, " + sysd["text"], "input": INPUT_TEXT,
            "num_orb": 2 * sysd["M"], "num_e": sysd["ne"], "Nd": nd, "input_dets": int(input_dets),
            "l2": "inputs larger than L2: the terms of one product are hundreds of GB against 129 MB of L2"}


def input_on_gpu(sg, path, sysd, nd):
    """v2 = top-Nd(H v1), v1 = H|HF>, both normalised, built by the device product
    on a construction context whose post-merge cut keeps every term."""
    c0 = sg.Context(path, 2 * sysd["M"], sysd["ne"], Nd=nd, coeff_cut=-1.0)
    hf = c0.vec(1)
    hf.upload(hf_key(sysd), np.array([1.0]))
    C1 = connected_per_det(sysd["M"], sysd["ne"] // 2, sysd["ne"] // 2) + 1
    m1, m2 = input_ms(sysd)
    v = c0.vec(C1)
    c0.SpMVMtply_bucket(hf, v, 0.0, 1.0)
    for m, cap in ((m1, HPSI_CAP), (m2, nd)):
        vm = c0.vec(m)
        vm.shrinkFrom(v)  # top m by |amplitude|, ties kept from the highest keys
        vm.normalize()
        v = c0.vec(cap)
        c0.SpMVMtply_bucket(vm, v, 0.0, 1.0)
    v.normalize()
    k, a = v.download()
    del v, vm, hf, c0
    return k, a


def input_on_cpu(be, sysd, nd):
    """The same construction with the CPU restatement (cut switched off, then restored)."""
    C1 = connected_per_det(sysd["M"], sysd["ne"] // 2, sysd["ne"] // 2) + 1
    be.set_cut(-1.0)
    try:
        m1, m2 = input_ms(sysd)
        k, a, _ = be.spmspv(hf_key(sysd), np.array([1.0]), C1, 0.0, 1.0)
        for m, cap in ((m1, HPSI_CAP), (m2, nd)):
            k, a = be.shrink_from(k, a, m)  # ties kept from the highest keys
            a = a / np.linalg.norm(a)
            k, a, _ = be.spmspv(k, a, cap, 0.0, 1.0)
        k2, a2 = k, a
    finally:
        be.set_cut(1e-5)
    return k2, a2 / np.linalg.norm(a2)


def top_slice(keys, amps, n):
    """The n largest |amplitude| entries (stable: ties keep the higher key), in key order."""
    order = np.argsort(-np.abs(amps), kind="stable")
    sel = np.sort(order[:n])
    return keys[sel], amps[sel]


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

def calibrate_sample(be, keys, amps, target_s, n0=100):
    """Largest top-n slice whose CPU product takes about target_s (at most the whole vector)."""
    n = n0
    while True:
        k, a = top_slice(keys, amps, n)
        t = time.perf_counter()
        be.spmspv(k, a, 10 ** 7, 0.0, 1.0)
        dt = time.perf_counter() - t
        if dt > target_s / 4 or n >= len(amps):
            return n, dt
        n = min(len(amps), int(n * min(8.0, max(2.0, target_s / max(dt, 1e-3) / 2))))


def cpu_baseline(sysd, path, keys, amps, target_s=15.0, threads=None):
    """The CPU restatement on all host threads, one product of a top-n slice of the
    GPU arm's input sized to ~target_s; returns the baseline and its product."""
    from oracle import oracle as orc
    orc.build_port()
    threads = threads or os.cpu_count() or 1
    be = orc.PortLib(words=key_words(sysd))
    be.setup(path, 2 * sysd["M"], sysd["ne"], 10 ** 7, nthread=threads)
    C = connected_per_det(sysd["M"], sysd["ne"] // 2, sysd["ne"] // 2)
    n, _ = calibrate_sample(be, keys, amps, target_s)
    k, a = top_slice(keys, amps, n)
    t = time.perf_counter()
    rk, ra, rd = be.spmspv(k, a, 10 ** 7, 0.0, 1.0)
    dt = time.perf_counter() - t
    base = {"value": n * C / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "top-%d determinants of the same input vector, one SpMSpV, %.1f s" % (n, dt),
            "seconds": dt, "dets": n}
    return base, (k, a), (rk, ra, rd)


def parity_report(ctx, sample, ref_out, cut=1e-5):
    """The GPU product of the slice cpu_baseline timed, against the CPU product."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from parity import compare_vectors
    k, a = sample
    rk, ra, rd = ref_out
    vin = ctx.vec_from(k, a)
    out = ctx.vec(10 ** 7)
    d = ctx.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    gk, ga = out.download()
    rep = {"sample_dets": int(len(a)), "against": "CPU restatement (oracle) product of the same slice",
           "diag_rel_diff": abs(d - rd) / max(abs(rd), 1e-300)}
    try:
        r = compare_vectors(rk, ra, gk, ga, cut=cut, capped=len(ra) == 10 ** 7)
        rep.update(ok=True, max_rel_diff=r["max_rel"], common_keys=r["common"],
                   edge_keys_only_cpu=r["edge_only_ref"], edge_keys_only_gpu=r["edge_only_got"],
                   tolerance="keys bit-exact off the 1e-5 cut edge; amplitudes 1e-12 relative, 1e-14 absolute")
    except AssertionError as e:
        rep.update(ok=False, error=str(e)[:300])
    rep["ok"] = bool(rep["ok"] and rep["diag_rel_diff"] <= 1e-12)
    del vin, out
    return rep


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
    keys, amps = input_on_cpu(be, sysd, args.nd)
    be.set_nd(10 ** 7)
    C = connected_per_det(sysd["M"], sysd["ne"] // 2, sysd["ne"] // 2)
    # each step: one product of the top-n slice, n sized for ~args.ref_step_s
    n, _ = calibrate_sample(be, keys, amps, args.ref_step_s, n0=200)
    ks, as_ = top_slice(keys, amps, n)
    for _ in range(args.warmup):
        be.spmspv(ks, as_, 10 ** 7, 0.0, 1.0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        be.spmspv(ks, as_, 10 ** 7, 0.0, 1.0)
    dt = (time.perf_counter() - t0) / args.steps
    val = n * C / dt
    cfg = bench_config(sysd, args.nd, len(amps))
    cfg["sample_dets"] = n
    out = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
           "parallelism": "CPU, %d threads" % threads,
           "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": "top-%d determinants of the input vector, one SpMSpV per step" % n},
           "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_gpu(args, rank, ws, local, dist):
    import sfci_gb300 as sg
    sg.load_library()
    sysd = SYSTEMS[args.config]
    path = workload_in(sysd)
    nd = args.nd
    M, NE, W = sysd["M"], sysd["ne"], key_words(sysd)
    in_k, in_a = input_on_gpu(sg, path, sysd, nd)
    ctx = sg.Context(path, 2 * M, NE, Nd=nd, hpsi_cap=HPSI_CAP, mem_budget=args.mem_budget, coeff_cut=args.cut)
    if args.class_passes is not None:
        ctx.set_class_passes(args.class_passes)
    vin = ctx.vec_from(in_k, in_a, cap=nd)
    n_in = vin.len
    out = ctx.vec(args.out_cap or HPSI_CAP)
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
    if args.profile_region:  # an ncu run with --profile-from-start off captures the timed steps only
        import torch
        torch.cuda.synchronize()
        torch.cuda.cudart().cudaProfilerStart()
    ctx.event_record(0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        diag = ctx.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    ctx.event_record(1)
    if args.profile_region:
        torch.cuda.synchronize()
        torch.cuda.cudart().cudaProfilerStop()
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
    keys_h, amps_h = in_k, in_a
    if args.no_e2e:
        return _finish_gpu(args, rank, ws, dist, ctx, sysd, path, nd, M, NE, W, n_in, C, T_conn, ms_max, clk, prof,
                           stats, out_len, launches, diag, keys_h, amps_h, None, 0, 0)
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
    return _finish_gpu(args, rank, ws, dist, ctx, sysd, path, nd, M, NE, W, n_in, C, T_conn, ms_max, clk, prof, stats,
                       out_len, launches, diag, keys_h, amps_h, e2e_s, h2d, d2h)


def _finish_gpu(args, rank, ws, dist, ctx, sysd, path, nd, M, NE, W, n_in, C, T_conn, ms_max, clk, prof, stats,
                out_len, launches, diag, keys_h, amps_h, e2e_s, h2d, d2h):
    tbytes = 8 * W + 8  # one determinant: key words + FP64 amplitude
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
    # the launches of one 56-orbital Nd=1e4 SpMSpV in one generation pass, 2 partition levels, 8 GB device
    # budget: level buffers well above L2), scaled here to a launch by the terms it processes
    ncu_bytes_per_term = {"scatter": 26.31, "partition": 38.50 * levels, "merge": 16.07}
    dom = max(prof, key=lambda k: prof[k][0])
    dms, dl = prof[dom]
    per_launch_bytes = alg[dom] / max(dl, 1)
    per_launch_ms = dms / max(dl, 1)
    achieved = per_launch_bytes / (per_launch_ms * 1e-3) / 1e9 if per_launch_ms > 0 else 0.0
    traffic = (ncu_bytes_per_term[dom] * T * args.steps / max(dl, 1)) if (dom in ncu_bytes_per_term and W == 1) \
        else None  # measured for one-word keys
    value = T_conn * ws / (ms_max * 1e-3)
    e2e_val = T_conn * ws / e2e_s if e2e_s else None
    # the whole product under the materialise-once model: read the input, write
    # and read every connected term once, write the merged determinants once
    B = (n_in + 2 * T_conn + stats["unique"]) * tbytes
    prod_ach = B / (ms_max * 1e-3) / 1e9
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max, "s_per_iter": ms_max / 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(sysd, nd, n_in),
        "parallelism": "replicas" if ws > 1 else "1 GPU",
        "stats": {"connected_per_det": C, "emitted_per_det_reference": emitted_per_det(M, NE // 2, NE // 2),
                  "generated_terms_per_step": T, "merged_unique_per_step": stats["unique"],
                  "survivors_per_step": surv, "output_dets": out_len, "passes": stats["passes"],
                  "leaves": stats["leaves"], "partition_levels": levels,
                  "terms_gb_per_step": tbytes * T / 1e9},
        "roofline": {"bound": "hbm", "kernel": kernels[dom], "phase": dom, "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "peak_source": how, "traffic": traffic,
                     "traffic_unit": "bytes per launch", "algorithmic_bytes_per_launch": per_launch_bytes,
                     "launches": dl, "ms_per_launch": per_launch_ms},
        "product_roofline": {"bytes_model": "(Nd + 2*T_conn + U) * (K + 8)", "bytes_per_step": B,
                             "achieved": prod_ach, "peak": hbm, "unit": "GB/s", "frac": prod_ach / hbm,
                             "peak_source": how},
        "phases_ms_per_step": {k: v[0] / args.steps for k, v in prof.items()},
        "e2e": ({"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                 "ms_per_step": e2e_s * 1e3} if e2e_s else None),
        "gpu_launches": launches,
        "clocks": clk,
        "diag": diag,
    }
    if not args.no_cpu_baseline:
        base, sample, ref_out = cpu_baseline(sysd, path, keys_h, amps_h, target_s=args.cpu_seconds)
        res["cpu_baseline"] = base
        ctx.trim()  # the timed product's scratch holds most of the device
        res["parity"] = parity_report(ctx, sample, ref_out)
    print(json.dumps(res), flush=True)
    barrier(dist)


# ---------------------------------------------------------------------------
# learned excitation screen: train on logged labels, then plain vs screened
# ---------------------------------------------------------------------------

def _krylov_input(sg, ctx, sysd, nd, cap=HPSI_CAP):
    """top-nd of H (H|HF>) with the product's own cut, normalised (the sources a
    Lanczos step would multiply)."""
    hf = ctx.vec(1)
    hf.upload(hf_key(sysd), np.array([1.0]))
    v1 = ctx.vec(cap)
    ctx.SpMVMtply_bucket(hf, v1, 0.0, 1.0)
    v1.normalize()
    w = ctx.vec(cap)
    ctx.SpMVMtply_bucket(v1, w, 0.0, 1.0)
    v2 = ctx.vec(nd)
    v2.shrinkFrom(w)
    v2.normalize()
    return v2


def run_screen(args):
    """Screen study: labels from plain products on 112-spin-orbital, 18-electron
    synthetic RHF systems of seeds 6-9, Adam training of the MLP on them, then the
    truncated Lanczos driver on the seed-5 system with and without the screen
    (threshold, guard, and floor at the labels' minimum term).  The energy of
    every run is judged by the unscreened calc_energy of its final vector; a
    screened run is accepted when it is within tol of the plain one."""
    import sfci_gb300 as sg
    sg.load_library()
    M, NE = 56, 18
    train_seeds = [6, 7, 8, 9]
    res = {"metric": METRIC, "unit": "s (time to energy)", "higher_is_better": False, "mode": "learned screen",
           "dtype": "f64 products, bf16 MLP (fp32 accumulate)", "data": "synthetic"}
    t0 = time.perf_counter()
    tr = {"systems": [], "examples": 0, "positives": 0}
    scr = None
    ctxs = []
    for sd in train_seeds:
        sysd = dict(M=M, ne=NE, seeds=(sd,), text="")
        path = workload_in(sysd)
        ctx = sg.Context(path, 2 * M, NE, Nd=args.screen_log_nd, hpsi_cap=HPSI_CAP)
        ctxs.append(ctx)
        if scr is None:
            scr = sg.Screen(ctx, seed=1)
        vin = _krylov_input(sg, ctx, sysd, args.screen_log_nd)
        out = ctx.vec(HPSI_CAP)
        ctx.SpMVMtply_bucket(vin, out, 0.0, 1.0)
        # the screen lives on the first context; each system logs from its own.
        # A group is alive when a term above 1e-3 of the cut lands on a survivor.
        ne, npos = scr.log(vin, out, min_term=args.screen_min_term)
        tr["systems"].append({"seed": sd, "sources": vin.len, "examples": ne, "positives": npos})
        tr["examples"] += ne
        tr["positives"] += npos
        del vin, out
        ctx.trim()
        if len(ctxs) > 1:
            ctxs.pop()
            del ctx
    pos_frac = tr["positives"] / max(tr["examples"], 1)
    pw = min(20.0, max(1.0, 0.25 * (1 - pos_frac) / max(pos_frac, 1e-9)))
    t1 = time.perf_counter()
    losses = []
    steps_done = 0
    while steps_done < args.screen_steps:
        n = min(500, args.screen_steps - steps_done)
        losses.append(scr.train(n, batch_tiles=64, lr=args.screen_lr, pos_weight=pw))
        steps_done += n
    t2 = time.perf_counter()
    tr.update(positive_fraction=pos_frac, pos_weight=pw, steps=steps_done, batch=64 * 128,
              loss_curve=losses, log_seconds=t1 - t0, train_seconds=t2 - t1)
    res["training"] = tr
    # evaluation system: seed 5; the screen's weights are moved to a context on it
    sysd = dict(M=M, ne=NE, seeds=(args.screen_seed,), text="")
    path = workload_in(sysd)
    params = scr.params()
    del scr
    ctxs.clear()
    ev = sg.Context(path, 2 * M, NE, Nd=args.screen_nd, hpsi_cap=HPSI_CAP)
    scr_e = sg.Screen(ev, seed=1)
    scr_e.set_params(params)
    runs = []

    def lanczos(thr, guard=0.0, floor=0.0):
        ev.set_screen(None if thr is None else scr_e, 0.0 if thr is None else thr, guard, floor)
        st0 = ev.screen_stats()
        v = ev.vec(args.screen_nd)
        v.upload(hf_key(sysd), np.array([1.0]))
        ev.profile(False)
        ta = time.perf_counter()
        en, fe = ev.sparse_krylov_solve_eigenval(v, args.screen_nl, 1)
        tb = time.perf_counter()
        st1 = ev.screen_stats()
        d = {k: st1[k] - st0[k] for k in st1}
        return {"threshold": thr, "guard": guard, "floor": floor, "seconds": tb - ta, "gsaes_energy": float(en[0]),
                "energy": fe,
                "kept_group_fraction": d["kept_groups"] / d["groups"] if d["groups"] else 1.0,
                "skipped_term_fraction": 1.0 - d["kept_terms"] / d["all_terms"] if d["all_terms"] else 0.0,
                "products": d["products"], "kept_terms": d["kept_terms"], "all_double_terms": d["all_terms"]}

    lanczos(None)  # warm-up (scratch allocation)
    plain = lanczos(None)
    C = connected_per_det(M, NE // 2, NE // 2)
    runs.append(plain)
    best = None
    t0_ = args.screen_thresholds[0]
    grid = [(t, 0.0, 0.0) for t in args.screen_thresholds] + [(t0_, gd, 0.0) for gd in args.screen_guards] + \
        [(t0_, gd, args.screen_min_term) for gd in args.screen_guards if gd > args.screen_min_term]
    for thr, guard, floor in grid:
        r = lanczos(thr, guard, floor)
        r["dE"] = r["energy"] - plain["energy"]
        runs.append(r)
        if abs(r["dE"]) <= args.screen_tol and (best is None or r["seconds"] < best["seconds"]):
            best = r
    res["config"] = {"workload": "truncated Lanczos, 112 spin orbitals, 18 electrons, synthetic RHF seed %d"
                                 % args.screen_seed, "num_orb": 2 * M, "num_e": NE, "Nd": args.screen_nd,
                     "Nl": args.screen_nl, "restarts": 1, "train_seeds": train_seeds,
                     "log_Nd": args.screen_log_nd, "tol_Eh": args.screen_tol}
    res["runs"] = runs
    res["plain_seconds"] = plain["seconds"]
    res["chosen"] = best
    res["value"] = best["seconds"] if best else plain["seconds"]
    res["speedup_vs_plain"] = plain["seconds"] / best["seconds"] if best else 1.0
    res["fallback"] = best is None
    res["connected_per_det"] = C
    print(json.dumps(res), flush=True)


def run_lanczos(args):
    """The whole truncated Lanczos ground-state solve of the selected system
    (sparse_krylov_solve_eigenval as the sfci binary runs it, from |HF>):
    wall time, products, time per Krylov iteration and the energies."""
    import sfci_gb300 as sg
    sg.load_library()
    sysd = SYSTEMS[args.config]
    path = workload_in(sysd)
    M, NE = sysd["M"], sysd["ne"]
    ctx = sg.Context(path, 2 * M, NE, Nd=args.nd, hpsi_cap=HPSI_CAP)
    v = ctx.vec(args.nd)
    v.upload(hf_key(sysd), np.array([1.0]))
    l0 = ctx.launches()
    t0 = time.perf_counter()
    en, fe = ctx.sparse_krylov_solve_eigenval(v, args.lanczos_nl, args.lanczos_restarts)
    t = time.perf_counter() - t0
    done = int(np.sum(~np.isnan(en)))
    products = done * args.lanczos_nl
    res = {"metric": METRIC, "mode": "truncated Lanczos solve", "unit": "s",
           "config": {"workload": "sparse_krylov_solve_eigenval from |HF>, " + sysd["text"], "num_orb": 2 * M,
                      "num_e": NE, "Nd": args.nd, "Nl": args.lanczos_nl, "num_restart": args.lanczos_restarts},
           "value": t, "higher_is_better": False, "restarts_run": done, "products": products,
           "s_per_krylov_iteration": t / max(products, 1), "energies": [float(x) for x in en[~np.isnan(en)]],
           "final_energy": fe, "gpu_launches": ctx.launches() - l0, "dtype": "f64", "data": "synthetic"}
    print(json.dumps(res), flush=True)


def run_mlp(args):
    """Throughput of the screen's tensor-core kernels on the 56-spin-orbital
    system: inference over every term group of a Krylov vector's top
    --mlp-sources determinants (1,870 groups each), and Adam training steps on
    the groups' labels.  Tensor FLOPs as the MMAs execute them: per group for
    inference 2 x 256 x (512 + 256) (layer 1's 0/1 rows: occupancy, p, q, r;
    and layer 2); per training example the forward and backward 256 x 256
    products and the weight-gradient products of both layers
    (2 x 256 x (256 + 256 + 576))."""
    import sfci_gb300 as sg
    sg.load_library()
    sysd = SYSTEMS[1]
    path = workload_in(sysd)
    M, NE = sysd["M"], sysd["ne"]
    cap = args.out_cap or HPSI_CAP
    ctx = sg.Context(path, 2 * M, NE, Nd=args.mlp_sources, hpsi_cap=cap, mem_budget=args.mem_budget)
    vin = _krylov_input(sg, ctx, sysd, args.mlp_sources, cap)
    scr = sg.Screen(ctx, seed=3)
    out = ctx.vec(cap)
    ctx.SpMVMtply_bucket(vin, out, 0.0, 1.0)
    ne, npos = scr.log(vin, out)
    scr.predict(vin, 0.5)  # warm-up
    t0 = time.perf_counter()
    reps = 5
    for _ in range(reps):
        r = scr.predict(vin, 0.5)
    t_inf = (time.perf_counter() - t0) / reps
    groups = r["groups"]
    scr.train(2, batch_tiles=args.mlp_batch_tiles, lr=1e-3)  # warm-up
    steps = 50
    t0 = time.perf_counter()
    scr.train(steps, batch_tiles=args.mlp_batch_tiles, lr=1e-3)
    t_tr = (time.perf_counter() - t0) / steps
    B = args.mlp_batch_tiles * 128
    f_inf = 2.0 * 256 * (512 + 256) * groups
    f_tr = 2.0 * 256 * (256 + 256 + 256 + 576) * B
    peak = None
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peak = float(json.load(f)["bf16_tflops"])
    except Exception:
        pass
    res = {"metric": METRIC, "mode": "screen MLP throughput", "unit": "tensor TFLOP/s",
           "config": {"workload": "MLP 576-256-256-1 on the term groups of a 56-spin-orbital Krylov vector",
                      "sources": vin.len, "groups": groups, "batch": B},
           "inference": {"seconds": t_inf, "groups_per_s": groups / t_inf, "tflops": f_inf / t_inf / 1e12,
                         "frac_of_bf16_peak": (f_inf / t_inf / 1e12 / peak) if peak else None},
           "training": {"seconds_per_step": t_tr, "examples_per_s": B / t_tr, "tflops": f_tr / t_tr / 1e12,
                        "frac_of_bf16_peak": (f_tr / t_tr / 1e12 / peak) if peak else None},
           "logged": {"examples": ne, "positives": npos}, "bf16_peak_tflops": peak}
    print(json.dumps(res), flush=True)


def run_batch(args):
    """Batched bond-stretch curve: 32 instances (seed-4 synthetic RHF integrals
    interpolated in t, 40-80 spin orbitals, 10-16 electrons, Nd geometric from
    1e5 to 2e6 times --batch-scale), advanced together by the batched Lanczos
    driver (one product over all instances per Krylov step), against the 32
    unbatched runs one after another.  The product plan is autotuned on the
    largest instance first."""
    import sfci_gb300 as sg
    from sfci_gb300 import fcidump as fd
    sg.load_library()
    curve = fd.bond_stretch_curve(32, 4, args.batch_scale)
    d = os.path.join(tempfile.gettempdir(), "sfci_bench", "curve")
    os.makedirs(d, exist_ok=True)
    paths = []
    t0 = time.perf_counter()
    for k, inst in enumerate(curve):
        p = os.path.join(d, "c%02d_m%d_ne%d_IN" % (k, inst["num_orb"] // 2, inst["num_e"]))
        if not os.path.exists(p):
            fd.bond_stretch_to_in_file(p + ".tmp", inst["num_orb"] // 2, inst["num_e"], 4, inst["t"])
            os.replace(p + ".tmp", p)
        paths.append(p)
    t_files = time.perf_counter() - t0
    Nl, R = args.batch_nl, 1
    orbs = [x["num_orb"] for x in curve]
    nes = [x["num_e"] for x in curve]
    # hpsi_cap is per instance in the batched driver: the same cap as the unbatched runs
    bc = sg.Context.batch(paths, orbs, nes, Nd=10 ** 9, hpsi_cap=HPSI_CAP)
    # autotune on the largest instance's two-step vector, in the batched context
    big = len(curve) - 1
    hf = bc.vec(1)
    hf.upload(sg.tag_keys(np.array([[(1 << nes[big]) - 1, 0]], np.uint64), big), np.array([1.0]))
    w = bc.vec(HPSI_CAP)
    bc.SpMVMtply_bucket(hf, w, 0.0, 1.0)
    w.normalize()
    v2 = bc.vec(curve[big]["Nd"])
    tmp = bc.vec(HPSI_CAP)
    bc.SpMVMtply_bucket(w, tmp, 0.0, 1.0)
    v2.shrinkFrom(tmp)
    v2.normalize()
    plan, plan_ms = bc.autotune(v2, tmp)
    del hf, w, v2, tmp

    def start_vectors(ctx, tagged):
        vs = []
        for k, inst in enumerate(curve):
            v = ctx.vec(inst["Nd"])
            key = np.array([[(1 << inst["num_e"]) - 1, 0]], np.uint64)
            v.upload(sg.tag_keys(key, k) if tagged else key, np.array([1.0]))
            vs.append(v)
        return vs

    bc.batch_lanczos(start_vectors(bc, True), 2, 1)  # warm-up: scratch allocation
    vs = start_vectors(bc, True)
    l0 = bc.launches()
    bc.profile(True)
    bc.profile_reset()
    tb0 = time.perf_counter()
    en_b, fe_b = bc.batch_lanczos(vs, Nl, R)
    t_batched = time.perf_counter() - tb0
    prof_b = {k: v[0] for k, v in bc.profile_read().items()}
    bc.profile(False)
    launches_b = bc.launches() - l0
    plan_b = bc.tuning()
    bc.trim()
    # unbatched: every instance in its own context, one after another
    en_u, fe_u, t_un = [], [], 0.0
    launches_u = 0
    prof_u = {}
    for k, inst in enumerate(curve):
        c = sg.Context(paths[k], inst["num_orb"], inst["num_e"], Nd=inst["Nd"], hpsi_cap=HPSI_CAP)
        c.set_tuning(**plan_b)
        v = c.vec(inst["Nd"])
        v.upload(sg.keys_from_ints([(1 << inst["num_e"]) - 1], c.words), np.array([1.0]))
        l0 = c.launches()
        c.profile(True)
        ta = time.perf_counter()
        e, f = c.sparse_krylov_solve_eigenval(v, Nl, R)
        t_un += time.perf_counter() - ta
        for kk, vv in c.profile_read().items():
            prof_u[kk] = prof_u.get(kk, 0.0) + vv[0]
        launches_u += c.launches() - l0
        en_u.append(e)
        fe_u.append(f)
        del v, c
    dE = [float(abs(fe_b[k] - fe_u[k])) for k in range(len(curve))]
    dG = [float(np.nanmax(np.abs(en_b[k] - en_u[k]))) for k in range(len(curve))]
    res = {"metric": METRIC, "mode": "batched bond-stretch curve", "unit": "s per batched Lanczos run",
           "value": t_batched, "higher_is_better": False, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "32-instance bond-stretch curve, seed-4 synthetic RHF interpolated in t "
                                  "(off-diagonal x(1+3t), diagonal gap x(1-0.6t))",
                      "num_orb": [min(orbs), max(orbs)], "num_e": [min(nes), max(nes)],
                      "Nd": [curve[0]["Nd"], curve[-1]["Nd"]], "Nd_scale": args.batch_scale, "Nl": Nl,
                      "restarts": R},
           "instances": [{"t": x["t"], "num_orb": x["num_orb"], "num_e": x["num_e"], "Nd": x["Nd"],
                          "energy": float(fe_b[k]), "dE_vs_unbatched": dE[k], "dE_gsaes": dG[k]}
                         for k, x in enumerate(curve)],
           "max_dE_vs_unbatched": max(dE), "max_dE_gsaes": max(dG),
           "batched_seconds": t_batched, "unbatched_seconds": t_un, "speedup": t_un / t_batched,
           "gpu_launches": {"batched": launches_b, "unbatched": launches_u},
           "product_phase_ms": {"batched": prof_b, "unbatched": prof_u},
           "autotune": {"plan": plan_b, "ms": plan_ms}, "files_seconds": t_files}
    print(json.dumps(res), flush=True)


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
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end (host buffer) leg")
    ap.add_argument("--class-passes", type=int, default=None, choices=[-1, 0, 1],
                    help="generation passes by target alpha class: 0 when needed (default), 1 always, -1 never")
    ap.add_argument("--profile-region", action="store_true",
                    help="bracket the timed steps with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--cut", type=float, default=1e-5,
                    help="post-merge cut of the timed product (profiling: a smaller cut gives more survivors)")
    ap.add_argument("--out-cap", type=int, default=0,
                    help="capacity of the product's output (profiling: a cap below the survivors runs the "
                         "radix select and compaction)")
    ap.add_argument("--mem-budget", type=int, default=0,
                    help="device bytes the SpMSpV may use (0: 80%% of free); a small budget forces several "
                         "generation passes on a small case, e.g. for profiling")
    ap.add_argument("--screen", action="store_true",
                    help="learned-screen study (112 spin orbitals): train, then plain vs screened Lanczos")
    ap.add_argument("--screen-nd", type=int, default=200000)
    ap.add_argument("--screen-nl", type=int, default=8)
    ap.add_argument("--screen-log-nd", type=int, default=1800)
    ap.add_argument("--screen-steps", type=int, default=3000)
    ap.add_argument("--screen-lr", type=float, default=1e-3)
    ap.add_argument("--screen-seed", type=int, default=5)
    ap.add_argument("--screen-tol", type=float, default=1e-5)
    ap.add_argument("--screen-min-term", type=float, default=1e-8)
    ap.add_argument("--screen-thresholds", type=float, nargs="+", default=[0.01])
    ap.add_argument("--screen-guards", type=float, nargs="*", default=[1e-5, 1e-6, 1e-7],
                    help="guards tried with the first threshold: groups with |c_j| max|V| >= guard always kept; "
                         "each is tried again with the floor at the labels' minimum term")
    ap.add_argument("--batch", action="store_true",
                    help="batched bond-stretch curve: 32 instances, batched vs unbatched Lanczos")
    ap.add_argument("--batch-scale", type=float, default=0.01,
                    help="scale of the instances' Nd (1.0: 1e5 to 2e6)")
    ap.add_argument("--batch-nl", type=int, default=10)
    ap.add_argument("--mlp", action="store_true", help="throughput of the screen's tensor-core MLP kernels")
    ap.add_argument("--mlp-sources", type=int, default=20000)
    ap.add_argument("--mlp-batch-tiles", type=int, default=128)
    ap.add_argument("--lanczos", action="store_true", help="the whole truncated Lanczos solve (time per iteration)")
    ap.add_argument("--lanczos-nl", type=int, default=30)
    ap.add_argument("--lanczos-restarts", type=int, default=4)
    args = ap.parse_args()
    if args.lanczos:
        run_lanczos(args)
        return
    if args.mlp:
        run_mlp(args)
        return
    if args.screen:
        run_screen(args)
        return
    if args.batch:
        run_batch(args)
        return
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
