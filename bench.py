"""Benchmark of the SkelCL skeleton path on one GB300.

Headline workload (one "step"): inclusive Scan(int32 add) over N = 2^28 values
uniform in {0..1000} (seed 0), then Map(x -> x mod 7919) in place -- the
integer scan + map configuration.  The inclusive scan is the library's
SCL_SHAPE_INCLUSIVE form of the reference's exclusive Scan (= exclusive (+) x).

  value      algorithmic HBM bytes / s over the timed steps, inputs resident
             in HBM (scan 2*4N + map 2*4N bytes per step)
  e2e        the same metric through the C ABI with pinned HOST buffers: every
             step copies the input in and the result out
  roofline   the dominant kernel (the scan) against the measured HBM copy
             bandwidth (MEASURED_PEAKS.json)
  skeletons  secondary per-skeleton figures (dot product, float scan and its
             adjoint, MapOverlap 8192^2 R=5, AllPairs 8192x4096x8192,
             Manhattan AllPairs), each against its own roofline

--impl reference times the CPU restatement of the same workload (the
reference SkelCL needs an OpenCL platform and libclang, neither of which
exists on this pool) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_SCAN = 1 << 28
MOD = 7919
BYTES_SCAN = 2 * 4 * N_SCAN
BYTES_MAP = 2 * 4 * N_SCAN
METRIC = "HBM GB/s (int32 inclusive Scan + Map(x mod 7919), N=2^28)"
WORKLOAD = "inclusive Scan(int32 +) over 2^28 then Map(x mod 7919)"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), float(d.get("bf16_tflops", 1876.6)), "measured"
    return 6800.0, 1900.0, "fallback"


def traffic_table():
    """Per-launch DRAM bytes from the committed ncu summaries (kernel -> bytes)."""
    t = {}
    p = ROOT / "profiles" / "traffic_per_launch.txt"
    if p.exists():
        for line in p.read_text().splitlines():
            line = line.split("#", 1)[0].strip()
            if line:
                k, v = line.split()[:2]
                t[k] = float(v)
    return t


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(value: float, dist) -> float:
    """The slowest rank's time (replicas run the same work: the job takes as
    long as its slowest GPU).  `dist` is torch.distributed or None."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def timed(S, fn, steps: int, warmup: int, kernel_events=None):
    """Warm-up, then time exactly `steps` calls of fn with events on the
    library stream (synchronised on both sides)."""
    for _ in range(warmup):
        fn()
    S.sync()
    e0, e1 = S.Event(), S.Event()
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    S.sync()
    return e0.elapsed_ms(e1) / steps


def run_gpu(args):
    import oracle
    import skelcl_gb300 as S

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # barrier + max over ranks only
        dist.init_process_group("gloo", init_method="env://")
    S.init(local_rank if world > 1 else 0)
    hbm_peak, bf16_peak, peak_kind = peaks()

    # ---- headline: scan + map over 2^28 int32 ------------------------------------
    x = oracle.mod_i32(N_SCAN, 0, 1001)
    scan = S.Program(S.KIND_SCAN, "int func(int x, int y){ return x+y; }", ["int"], identity="0")
    mod = S.Program(S.KIND_MAP, "int func(int x){ return x % 7919; }", ["int", "int"])
    dx = S.DeviceArray.from_numpy(x)
    dy = S.DeviceArray(N_SCAN, np.int32)

    ev = [S.Event() for _ in range(3)]
    per_kernel = {"scan": [], "map": []}

    def step():
        scan.launch([dx, dy], n=N_SCAN, flags=S.SHAPE_INCLUSIVE)
        mod.launch([dy, dy], n=N_SCAN)

    def step_events():
        ev[0].record()
        scan.launch([dx, dy], n=N_SCAN, flags=S.SHAPE_INCLUSIVE)
        ev[1].record()
        mod.launch([dy, dy], n=N_SCAN)
        ev[2].record()

    for _ in range(args.warmup):
        step()
    S.sync()
    # correctness of the measured configuration (bit-exact vs the oracle, sampled)
    got = dy.to_numpy()
    ref = oracle.scan_incl_mod_i32_mt(x, MOD)
    parity = bool(np.array_equal(got, ref))
    del got, ref

    if dist:
        dist.barrier()
    sampler = ClockSampler(local_rank)
    sampler.start()
    launches0 = S.launch_count()
    t0 = S.Event()
    t1 = S.Event()
    S.sync()
    evs = [[S.Event() for _ in range(3)] for _ in range(args.steps)]
    t0.record()
    for k in range(args.steps):
        ev[:] = evs[k]
        step_events()
    t1.record()
    S.sync()
    ms_total = t0.elapsed_ms(t1)
    for e in evs:
        per_kernel["scan"].append(e[0].elapsed_ms(e[1]))
        per_kernel["map"].append(e[1].elapsed_ms(e[2]))
    launches = S.launch_count() - launches0
    clocks = sampler.stop()
    ms_step = max_over_ranks(ms_total / args.steps, dist)
    value = world * (BYTES_SCAN + BYTES_MAP) / (ms_step * 1e-3) / 1e9

    scan_ms = statistics.mean(per_kernel["scan"])
    map_ms = statistics.mean(per_kernel["map"])
    dominant = "scan" if scan_ms >= map_ms else "map"
    dom_ms = max(scan_ms, map_ms)
    dom_bytes = BYTES_SCAN if dominant == "scan" else BYTES_MAP
    achieved = dom_bytes / (dom_ms * 1e-3) / 1e9
    traffic = traffic_table()
    tkey = {"scan": "scan_int32_2^28", "map": "map_mod_int32_2^28"}[dominant]

    # ---- e2e through the C ABI with pinned host buffers -----------------------------
    # Every step copies its input in (copy stream 1), runs Scan + Map (stream
    # 0) and reads its result back (copy stream 2); two device buffer pairs
    # let step k's input copy overlap step k-1's read-back (the host link
    # carries ~0.2 TB/s each way, ~0.34 TB/s both ways at once).
    import ctypes
    L = S.lib()
    hin = ctypes.c_void_p()
    hout = ctypes.c_void_p()
    S.check(L.scl_host_alloc(4 * N_SCAN, ctypes.byref(hin)))
    S.check(L.scl_host_alloc(4 * N_SCAN, ctypes.byref(hout)))
    ctypes.memmove(hin, x.ctypes.data, 4 * N_SCAN)
    dxs = [dx, S.DeviceArray(N_SCAN, np.int32)]
    dys = [dy, S.DeviceArray(N_SCAN, np.int32)]
    ev_in = [S.Event(), S.Event()]
    ev_done = [S.Event(), S.Event()]
    ev_out = [S.Event(), S.Event()]

    def e2e_step(k):
        b = k % 2
        if k >= 2:
            ev_done[b].wait_on(1)  # step k-2 has read input buffer b
        S.check(L.scl_h2d_on(1, dxs[b].ptr, hin, 4 * N_SCAN))
        ev_in[b].record_on(1)
        ev_in[b].wait_on(0)
        if k >= 2:
            ev_out[b].wait_on(0)   # step k-2's result has left output buffer b
        scan.launch([dxs[b], dys[b]], n=N_SCAN, flags=S.SHAPE_INCLUSIVE)
        mod.launch([dys[b], dys[b]], n=N_SCAN)
        ev_done[b].record_on(0)
        ev_done[b].wait_on(2)
        S.check(L.scl_d2h_on(2, hout, dys[b].ptr, 4 * N_SCAN))
        ev_out[b].record_on(2)

    def e2e_run(steps):
        e0, e1 = S.Event(), S.Event()
        S.sync()
        e0.record_on(0)
        e0.wait_on(1)
        for k in range(steps):
            e2e_step(k)
        ev_out[(steps - 1) % 2].wait_on(0)
        e1.record_on(0)
        S.sync()
        return e0.elapsed_ms(e1) / steps

    e2e_run(2)  # warm-up
    e2e_steps = max(4, args.steps)
    e2e_ms = e2e_run(e2e_steps)
    hres = np.ctypeslib.as_array(ctypes.cast(hout, ctypes.POINTER(ctypes.c_int32)), shape=(N_SCAN,))
    e2e_parity = bool(np.array_equal(hres, dy.to_numpy()))
    e2e_val = (BYTES_SCAN + BYTES_MAP) / (e2e_ms * 1e-3) / 1e9
    del hres
    L.scl_host_free(hin)
    L.scl_host_free(hout)
    del dx, dy, dxs, dys

    line = {
        "metric": METRIC,
        "value": round(value, 2),
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms_step, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic (SplitMix64 seed 0, uniform {0..1000})",
        "config": {"workload": WORKLOAD,
                   "n": N_SCAN, "l2": "inputs (1 GiB) larger than L2; no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "parity": {"bit_exact_vs_oracle": parity},
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1),
                     "peak": hbm_peak, "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                     "peak_source": f"hbm_gbs of {peak_kind}",
                     "traffic": traffic.get(tkey), "algorithmic_bytes": dom_bytes,
                     "per_kernel_ms": {"scan": round(scan_ms, 4), "map": round(map_ms, 4)}},
        "e2e": {"value": round(e2e_val, 2), "unit": "GB/s", "h2d_bytes_per_step": 4 * N_SCAN,
                "d2h_bytes_per_step": 4 * N_SCAN, "ms_per_step": round(e2e_ms, 3), "steps": e2e_steps,
                "result_matches_device": e2e_parity,
                "note": "pinned host buffers; input copy, Scan+Map and result read-back of "
                        "consecutive steps overlap on three streams"},
        "gpu_launches": launches,
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sample=N_SCAN)
    if rank == 0 and not args.headline_only:
        line["skeletons"] = secondary(S, oracle, hbm_peak, args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def cpu_baseline(sample: int, reps: int = 3):
    """The oracle's multithreaded scan+mod on a bounded sample (host cores)."""
    import oracle
    x = oracle.mod_i32(sample, 0, 1001)
    out = np.empty_like(x)
    nt = oracle.threads()
    oracle.scan_incl_mod_i32_mt(x, MOD, nt, out)
    ts = []
    for _ in range(reps):
        t = time.perf_counter()
        oracle.scan_incl_mod_i32_mt(x, MOD, nt, out)
        ts.append(time.perf_counter() - t)
    sec = statistics.median(ts)
    whole = " (the whole workload)" if sample == N_SCAN else ""
    return {"value": round(16 * sample / sec / 1e9, 3), "unit": "GB/s", "cores": nt, "kind": "port",
            "sample": f"2^{sample.bit_length() - 1} int32{whole} per run (scan+mod fused, two-pass "
                      f"chunked), median of {reps}"}


def fp32_peak_measured(S, device: int = 0, seconds: float = 0.6):
    """FP32 CUDA-core peak of this GPU, measured: the library's probe of 16
    independent FMA chains per thread at 2048 threads per SM (scalar
    fma.rn.f32, then packed fma.rn.f32x2), each timed with events on the
    library stream for about `seconds`, the SM clock sampled meanwhile.  The
    peak is the faster form's rate."""
    L = S.lib()
    sink = S.DeviceArray(1 << 21, np.float32)
    res = {}
    import ctypes
    for name, packed in (("scalar_ffma", 0), ("packed_ffma2", 1)):
        flops = ctypes.c_uint64(0)
        iters = 4096

        def fn():
            S.check(L.scl_debug_fp32_peak(packed, iters, sink.ptr, 1 << 21, ctypes.byref(flops)))
        ms1 = timed(S, fn, 3, 2)
        reps = max(10, int(seconds * 1e3 / max(ms1, 1e-3)))
        sampler = ClockSampler(device)
        sampler.start()
        ms = timed(S, fn, reps, 2)
        clk = sampler.stop()
        res[name] = {"TFLOPs": round(flops.value / ms / 1e9, 2), "ms": round(ms, 4), "launches": reps,
                     "sm_mhz_median": clk.get("sm_mhz"), "clock_reasons": clk.get("reasons")}
    peak = max(v["TFLOPs"] for v in res.values())
    res["peak_TFLOPs"] = peak
    res["note"] = ("dense FP32 FMA rate this GPU sustained at the sampled clock; the CUDA-core "
                   "kernels' fp32_frac is against it")
    return peak, res


def secondary(S, oracle, hbm_peak, args):
    out = {}
    fp32_peak, out["fp32_peak_measured"] = fp32_peak_measured(S)
    bf16_peak = peaks()[1]
    # dot product: Zip(mult) then Reduce(add), N = 2^24
    n = 1 << 24
    a = oracle.uniform_f32(n, 0, -1.0, 1.0)
    b = oracle.uniform_f32(n, 1, -1.0, 1.0)
    zp = S.Program(S.KIND_ZIP, "float func(float x, float y){ return x*y; }", ["float"] * 3)
    rp = S.Program(S.KIND_REDUCE, "float func(float x, float y){ return x+y; }", ["float"], identity="0")
    da, db = S.DeviceArray.from_numpy(a), S.DeviceArray.from_numpy(b)
    dz, dr = S.DeviceArray(n, np.float32), S.DeviceArray(1, np.float32)
    zms = timed(S, lambda: zp.launch([da, db, dz], n=n), 20, 3)
    rms = timed(S, lambda: rp.launch([dz, dr], n=n), 20, 3)
    dot = float(dr.to_numpy()[0])
    ref = oracle.dot_f64(a, b)
    # fused Reduce(Zip(x, y)): one pass over x and y, no intermediate vector
    zr = S.Program(S.KIND_ZIP_REDUCE, "float func(float x, float y){ return x+y; }", ["float"] * 3,
                   source2="float m(float x, float y){ return x*y; }", func2="m", identity="0")
    fms = timed(S, lambda: zr.launch([da, db, dr], n=n), 20, 3)
    fdot = float(dr.to_numpy()[0])
    # the same with the inputs rotating through four pairs (1 GiB of inputs,
    # more than L2): consecutive iterations find nothing of theirs in L2, so
    # these are HBM figures
    pairs = [(da, db)] + [(S.DeviceArray.from_numpy(oracle.uniform_f32(n, 10 + 2 * k, -1.0, 1.0)),
                           S.DeviceArray.from_numpy(oracle.uniform_f32(n, 11 + 2 * k, -1.0, 1.0)))
                          for k in range(3)]
    zs = [dz] + [S.DeviceArray(n, np.float32) for _ in range(3)]
    it = {"k": 0}

    def rot(fn):
        def step():
            k = it["k"] = (it["k"] + 1) % 4
            fn(k)
        return step
    zms_h = timed(S, rot(lambda k: zp.launch([pairs[k][0], pairs[k][1], zs[k]], n=n)), 20, 4)
    rms_h = timed(S, rot(lambda k: rp.launch([zs[k], dr], n=n)), 20, 4)
    fms_h = timed(S, rot(lambda k: zr.launch([pairs[k][0], pairs[k][1], dr], n=n)), 20, 4)
    # the same three with plain launches (no programmatic stream serialization)
    prev = S.set_overlapped_launches(False)
    plain = {"zip_ms": timed(S, rot(lambda k: zp.launch([pairs[k][0], pairs[k][1], zs[k]], n=n)), 20, 4),
             "reduce_ms": timed(S, rot(lambda k: rp.launch([zs[k], dr], n=n)), 20, 4),
             "fused_ms": timed(S, rot(lambda k: zr.launch([pairs[k][0], pairs[k][1], dr], n=n)), 20, 4)}
    S.set_overlapped_launches(prev)
    del pairs, zs
    out["dot_product_2^24"] = {
        "zip_GBps": round(12 * n / zms / 1e6, 1), "reduce_GBps": round(4 * n / rms / 1e6, 1),
        "zip_frac": round(12 * n / zms / 1e6 / hbm_peak, 3),
        "reduce_frac": round(4 * n / rms / 1e6 / hbm_peak, 3),
        "rel_err_vs_fp64": abs(dot - ref) / abs(ref),
        "fused_zip_reduce": {"ms": round(fms, 4), "GBps": round(8 * n / fms / 1e6, 1),
                             "unfused_ms": round(zms + rms, 4), "speedup": round((zms + rms) / fms, 2),
                             "rel_err_vs_fp64": abs(fdot - ref) / abs(ref)},
        "hbm": {"zip_GBps": round(12 * n / zms_h / 1e6, 1), "zip_frac": round(12 * n / zms_h / 1e6 / hbm_peak, 3),
                "reduce_GBps": round(4 * n / rms_h / 1e6, 1),
                "reduce_frac": round(4 * n / rms_h / 1e6 / hbm_peak, 3),
                "fused_ms": round(fms_h, 4), "fused_GBps": round(8 * n / fms_h / 1e6, 1),
                "fused_frac": round(8 * n / fms_h / 1e6 / hbm_peak, 3),
                "unfused_ms": round(zms_h + rms_h, 4),
                "plain_launches": {k: round(v, 4) for k, v in plain.items()},
                "note": "inputs rotating through four pairs (1 GiB): no L2 reuse between iterations; "
                        "'plain_launches': the same without programmatic stream serialization"},
        "note": "top-level figures: the same 128 MiB of inputs every iteration (about L2 size, "
                "so they include L2 reuse); 'hbm': rotating inputs"}
    del da, db, dz, dr

    # Map / Zip / Reduce at 2^26 and their adjoints (the user's vector-Jacobian
    # products; the broadcast for Reduce(+))
    n = 1 << 26
    hx, hy, hg = (oracle.uniform_f32(n, 2, -1.0, 1.0), oracle.uniform_f32(n, 4, -1.0, 1.0),
                  oracle.uniform_f32(n, 3, -1.0, 1.0))
    xa, ya, ga = S.DeviceArray.from_numpy(hx), S.DeviceArray.from_numpy(hy), S.DeviceArray.from_numpy(hg)
    x64, y64, g64 = hx.astype(np.float64), hy.astype(np.float64), hg.astype(np.float64)

    def rel_err(dev_arr, ref):
        """largest element-wise relative error against the FP64 value"""
        got = dev_arr.to_numpy().astype(np.float64)
        den = np.abs(ref)
        return float(np.max(np.divide(np.abs(got - ref), den, out=np.zeros_like(den), where=den > 0)))
    o1, o2 = S.DeviceArray(n, np.float32), S.DeviceArray(n, np.float32)
    mp = S.Program(S.KIND_MAP, "float func(float x){ return x*x + 1.0f; }", ["float", "float"])
    mpa = S.Program(S.KIND_MAP_ADJOINT, "float d(float x, float g){ return 2.0f*x*g; }", ["float", "float"], func="d")
    zpf = S.Program(S.KIND_ZIP, "float func(float x, float y){ return x*y; }", ["float"] * 3)
    zpa = S.Program(S.KIND_ZIP_ADJOINT, "float dl(float x, float y, float g){ return y*g; }\n"
                    "float dr(float x, float y, float g){ return x*g; }", ["float"] * 3, func="dl", func2="dr")
    rpf = S.Program(S.KIND_REDUCE, "float func(float x, float y){ return x+y; }", ["float"], identity="0")
    L = S.lib()
    adj = {}
    for name, f_bytes, a_bytes, fwd_fn, adj_fn in (
            ("map_x*x+1", 8, 12, lambda: mp.launch([xa, o1], n=n), lambda: mpa.launch([xa, ga, o1], n=n)),
            ("zip_x*y", 12, 20, lambda: zpf.launch([xa, ya, o1], n=n),
             lambda: zpa.launch([xa, ya, ga, o1, o2], n=n)),
            ("reduce_sum", 4, 4, lambda: rpf.launch([xa, o2], n=n),
             lambda: S.check(L.scl_adjoint_broadcast(ga.ptr, o1.ptr, n, S.DTYPE_F32, 0)))):
        f_ms = timed(S, fwd_fn, 10, 3)
        a_ms = timed(S, adj_fn, 10, 3)
        # errors against FP64: forward output, then the adjoint's
        fwd_fn()
        if name == "map_x*x+1":
            errs = {"fwd": rel_err(o1, x64 * x64 + 1.0)}
            adj_fn()
            errs["adjoint"] = rel_err(o1, 2.0 * x64 * g64)
        elif name == "zip_x*y":
            errs = {"fwd": rel_err(o1, x64 * y64)}
            adj_fn()
            errs["adjoint_left"] = rel_err(o1, y64 * g64)
            errs["adjoint_right"] = rel_err(o2, x64 * g64)
        else:
            ref = oracle.sum_f64(hx)
            errs = {"fwd": abs(float(o2.to_numpy()[0]) - ref) / abs(ref)}
            adj_fn()
            errs["adjoint"] = rel_err(o1, np.full(n, g64[0]))
        adj[name] = {"fwd_GBps": round(f_bytes * n / f_ms / 1e6, 1),
                     "adjoint_GBps": round(a_bytes * n / a_ms / 1e6, 1),
                     "adjoint_frac": round(a_bytes * n / a_ms / 1e6 / hbm_peak, 3),
                     "fwd_plus_adjoint_over_fwd": round((f_ms + a_ms) / f_ms, 3),
                     "bytes_per_elem_fwd_adjoint": [f_bytes, a_bytes],
                     "max_rel_err_vs_fp64": errs}
    out["elementwise_adjoints_2^26"] = adj
    del xa, ya, ga, o1, o2, hx, hy, hg, x64, y64, g64

    # fused Map(Scan(x)) on the headline workload: the scanned vector is not written
    xs = oracle.mod_i32(N_SCAN, 0, 1001)
    dxs, dys = S.DeviceArray.from_numpy(xs), S.DeviceArray(N_SCAN, np.int32)
    sm = S.Program(S.KIND_SCAN_MAP, "int func(int x, int y){ return x+y; }", ["int", "int"],
                   source2="int m(int x){ return x % 7919; }", func2="m", identity="0")
    f_ms = timed(S, lambda: sm.launch([dxs, dys], n=N_SCAN, flags=S.SHAPE_INCLUSIVE), 10, 3)
    exact = bool(np.array_equal(dys.to_numpy(), oracle.scan_incl_mod_i32_mt(xs, MOD)))
    out["fused_scan_map_int32_2^28"] = {
        "ms": round(f_ms, 4), "GBps_moved": round(8 * N_SCAN / f_ms / 1e6, 1),
        "frac_of_hbm": round(8 * N_SCAN / f_ms / 1e6 / hbm_peak, 3), "bit_exact_vs_oracle": exact,
        "note": "reads x and writes the result once (8 bytes per element); the unfused "
                "headline pipeline moves 16"}
    del dxs, dys, xs

    # float scan 2^26 and its adjoint (reverse scan of the upstream gradient)
    n = 1 << 26
    xf = oracle.uniform_f32(n, 2, -1.0, 1.0)
    g = oracle.uniform_f32(n, 3, -1.0, 1.0)
    sp = S.Program(S.KIND_SCAN, "float func(float x, float y){ return x+y; }", ["float"], identity="0.0f")
    dxf, dg, dyf, dgx = (S.DeviceArray.from_numpy(xf), S.DeviceArray.from_numpy(g),
                         S.DeviceArray(n, np.float32), S.DeviceArray(n, np.float32))
    fwd = timed(S, lambda: sp.launch([dxf, dyf], n=n, flags=S.SHAPE_INCLUSIVE), 10, 3)
    bwd = timed(S, lambda: sp.launch([dg, dgx], n=n, flags=S.SHAPE_INCLUSIVE | S.SHAPE_REVERSE), 10, 3)
    yf = dyf.to_numpy().astype(np.float64)
    ref = oracle.scan_f64(xf, inclusive=True)
    out["float_scan_2^26"] = {
        "fwd_GBps": round(8 * n / fwd / 1e6, 1), "fwd_frac": round(8 * n / fwd / 1e6 / hbm_peak, 3),
        "adjoint_GBps": round(8 * n / bwd / 1e6, 1),
        "fwd_plus_adjoint_over_fwd": round((fwd + bwd) / fwd, 3),
        "max_abs_err_vs_fp64": float(np.abs(yf - ref).max()),
        "max_abs_prefix": float(np.abs(ref).max()),
        "note": "about 8 us per call is fixed (launch, ramp of the first wave's look-back), and the FP64 "
                "carries cost about 3 % (float carries: 3 us less at 2^26): 2^28 below"}
    del dxf, dg, dyf, dgx, yf, ref
    n4 = 1 << 28
    hx4 = oracle.uniform_f32(n4, 2, -1.0, 1.0)
    dxf, dyf = S.DeviceArray.from_numpy(hx4), S.DeviceArray(n4, np.float32)
    fwd4 = timed(S, lambda: sp.launch([dxf, dyf], n=n4, flags=S.SHAPE_INCLUSIVE), 10, 3)
    bwd4 = timed(S, lambda: sp.launch([dxf, dyf], n=n4, flags=S.SHAPE_INCLUSIVE | S.SHAPE_REVERSE), 10, 3)
    errs = {}
    for key, rev in (("fwd", False), ("adjoint", True)):
        sp.launch([dxf, dyf], n=n4, flags=S.SHAPE_INCLUSIVE | (S.SHAPE_REVERSE if rev else 0))
        ref = oracle.scan_f64(hx4, inclusive=True, reverse=rev)
        errs[key] = float(np.abs(dyf.to_numpy().astype(np.float64) - ref).max())
        errs[key + "_max_abs_prefix"] = float(np.abs(ref).max())
        del ref
    out["float_scan_2^28"] = {"fwd_GBps": round(8 * n4 / fwd4 / 1e6, 1),
                              "fwd_frac": round(8 * n4 / fwd4 / 1e6 / hbm_peak, 3),
                              "adjoint_GBps": round(8 * n4 / bwd4 / 1e6, 1),
                              "fwd_plus_adjoint_over_fwd": round((fwd4 + bwd4) / fwd4, 3),
                              "max_abs_err_vs_fp64": errs}
    del dxf, dyf, hx4

    # MapOverlap 8192^2, R = 5 Gaussian, both paddings
    rows = cols = 8192
    img = oracle.uniform_f32(rows * cols, 5, 0.0, 255.0)
    w = oracle.gaussian_weights(5, 2.0)
    src = ("float func(input_matrix_t img, __global float* w) { float s = 0.0f;"
           " for (int dy = -5; dy <= 5; ++dy) for (int dx = -5; dx <= 5; ++dx)"
           "  s += getData(img, dx, dy) * w[(dy + 5) * 11 + (dx + 5)]; return s; }")
    di, do, dw = S.DeviceArray.from_numpy(img), S.DeviceArray(rows * cols, np.float32), S.DeviceArray.from_numpy(w.ravel())
    # adjoint of the linear stencil: the zero-padded transposed stencil (flipped
    # weights), plus the edge fold for NEAREST
    dwt = S.DeviceArray.from_numpy(np.ascontiguousarray(w.reshape(11, 11)[::-1, ::-1]).ravel())
    dg = S.DeviceArray.from_numpy(oracle.uniform_f32(rows * cols, 6, -1.0, 1.0))
    adj_src = ("float adj(input_matrix_t g, __global const float* w) { float s = 0.0f;"
               " for (int dy = -5; dy <= 5; ++dy) for (int dx = -5; dx <= 5; ++dx)"
               "  s += w[(dy + 5) * 11 + (dx + 5)] * getData(g, dx, dy); return s; }")
    pa = S.Program(S.KIND_MAPOVERLAP, adj_src, ["float", "float"], func="adj", overlap_range=5,
                   padding=S.PAD_NEUTRAL, neutral="0.0f")
    mo = {}
    for name, pad in (("neutral", S.PAD_NEUTRAL), ("nearest", S.PAD_NEAREST)):
        p = S.Program(S.KIND_MAPOVERLAP, src, ["float", "float"], overlap_range=5, padding=pad, neutral="0")
        ms = timed(S, lambda: p.launch([di, do], rows=rows, cols=cols, extra=S.buffer(dw)), 10, 3)
        gbps = 8 * rows * cols / ms / 1e6
        tflops = 242 * rows * cols / ms / 1e9

        def adjoint():
            pa.launch([dg, do], rows=rows, cols=cols, extra=S.buffer(dwt))
            if pad == S.PAD_NEAREST:
                S.check(L.scl_mapoverlap_adjoint_edges(dg.ptr, dwt.ptr, do.ptr, rows, cols, 5))

        a_ms = timed(S, adjoint, 10, 3)
        p.launch([di, do], rows=rows, cols=cols, extra=S.buffer(dw))
        ref = oracle.stencil_f64(img.reshape(rows, cols), 5, w, pad, 0.0)
        err = float(np.abs(do.to_numpy().reshape(rows, cols) - ref).max())
        del ref
        mo[name] = {"max_abs_err_vs_fp64": err, "GBps": round(gbps, 1), "hbm_frac": round(gbps / hbm_peak, 3),
                    "TFLOPs": round(tflops, 2), "fp32_frac": round(tflops / fp32_peak, 3),
                    "variant": p.last_variant, "adjoint_ms": round(a_ms, 4), "fwd_ms": round(ms, 4),
                    "fwd_plus_adjoint_over_fwd": round((ms + a_ms) / ms, 3)}
    out["mapoverlap_8192^2_R5"] = mo
    del di, do, dw, dwt, dg

    # AllPairs 8192x4096 . 4096x8192 (mult/add), and Manhattan 4096x256 . 256x4096
    M, K, N = 8192, 4096, 8192
    A = oracle.normal_f32(M * K, 7)
    B = oracle.normal_f32(K * N, 8)
    ap = S.Program(S.KIND_ALLPAIRS, "float func(float x, float y){ return x+y; }", ["float"] * 3,
                   source2="float func(float x, float y){ return x*y; }", identity="0")
    dA, dB, dP = S.DeviceArray.from_numpy(A), S.DeviceArray.from_numpy(B), S.DeviceArray(M * N, np.float32)
    res = {}
    rows_chk = np.arange(0, M, M // 16)
    ref = oracle.gemm_f64(A.reshape(M, K)[rows_chk], B.reshape(K, N))
    # the tensor-core launches take 128 x 256 output tiles here (automatic
    # choice); "_128col" repeats the 6-product one with 128 x 128 tiles
    # (the tensor-core tiles are taken in groups of 16 tile rows; "_rowmajor"
    # repeats the 6-product launch in plain row-major tile order)
    for name, var, items, cols, group in (("fp32_simt", S.VARIANT_SIMT, 0, 0, 0),
                                          ("tc_3xbf16_6prod", S.VARIANT_TC3XBF16, 3, 0, 0),
                                          ("tc_3xbf16_6prod_rowmajor", S.VARIANT_TC3XBF16, 3, 0, 1),
                                          ("tc_3xbf16_6prod_128col", S.VARIANT_TC3XBF16, 3, 128, 0),
                                          ("tc_3xbf16_3prod", S.VARIANT_TC3XBF16, 2, 0, 0)):
        tun = S.Tuning(variant=var, items=items, tile_h=cols, workgroup=group)
        ms = timed(S, lambda: ap.launch([dA, dB, dP], rows=M, cols=N, dim=K, tuning=tun), 3, 1)
        P = dP.to_numpy().reshape(M, N)
        err = np.abs(P[rows_chk].astype(np.float64) - ref)
        res[name] = {"ms": round(ms, 3), "TFLOPs": round(2 * M * N * K / ms / 1e9, 2),
                     "variant": ap.last_variant,
                     # CUDA-core kernel: FP32 flops over the measured FP32 peak;
                     # tensor cores: the bf16 products' flops over the bf16 peak
                     "frac": round((2 * M * N * K if var == S.VARIANT_SIMT else
                                    (6 if items == 3 else 3) * 2 * M * N * K) / ms / 1e9 /
                                   (fp32_peak if var == S.VARIANT_SIMT else bf16_peak), 3),
                     "frac_of": "measured FP32 peak" if var == S.VARIANT_SIMT else
                                "bf16 burst peak (MEASURED_PEAKS.json), bf16 products' flops",
                     "normwise_err_vs_fp64": float(err.max() / np.abs(ref).max()),
                     "median_rel_err_vs_fp64": float(np.median(err / np.maximum(np.abs(ref), 1e-30)))}
    # the split pass alone (both operands into bf16 planes), which every
    # tensor-core launch above includes
    import ctypes
    for name, parts in (("tc_3xbf16_6prod", 3), ("tc_3xbf16_3prod", 2)):
        need = ctypes.c_size_t(0)
        S.check(S.lib().scl_debug_allpairs_split(None, None, M, N, K, parts, 0, None, 0, ctypes.byref(need)))
        scratch = S.DeviceArray((need.value + 15) // 16 * 4, np.float32)
        sms = timed(S, lambda: S.check(S.lib().scl_debug_allpairs_split(
            dA.ptr, dB.ptr, M, N, K, parts, 0, scratch.ptr, scratch.n * 4, None)), 5, 2)
        del scratch
        res[name]["split_ms"] = round(sms, 3)
        res[name]["contraction_ms"] = round(res[name]["ms"] - sms, 3)
        prods = 6 if parts == 3 else 3
        res[name]["contraction_frac_of_bf16_peak"] = round(
            prods * 2 * M * N * K / (res[name]["ms"] - sms) / 1e9 / bf16_peak, 3)
    res["speedup_tc6_over_simt"] = round(res["fp32_simt"]["ms"] / res["tc_3xbf16_6prod"]["ms"], 2)
    res["speedup_tc3_over_simt"] = round(res["fp32_simt"]["ms"] / res["tc_3xbf16_3prod"]["ms"], 2)
    # backward of L = sum(G * P) as two AllPairs on transposed operands (tensor cores)
    hG = oracle.normal_f32(M * N, 9).reshape(M, N)
    dG = S.DeviceArray.from_numpy(hG)
    dgA, dgB = S.DeviceArray(M * K, np.float32), S.DeviceArray(K * N, np.float32)
    f_ms = timed(S, lambda: ap.launch([dA, dB, dP], rows=M, cols=N, dim=K), 3, 1)
    a_ms = timed(S, lambda: ap.launch([dG, dB, dgA], rows=M, cols=K, dim=N, flags=S.SHAPE_TRANS_RIGHT), 3, 1)
    b_ms = timed(S, lambda: ap.launch([dA, dG, dgB], rows=K, cols=N, dim=M, flags=S.SHAPE_TRANS_LEFT), 3, 1)
    # normwise errors against FP64 on 16 sampled rows of dA = G B^T and dB = A^T G
    A2, B2 = A.reshape(M, K), B.reshape(K, N)
    ra, rb = np.arange(0, M, M // 16), np.arange(0, K, K // 16)
    ref_a = oracle.gemm_f64(np.ascontiguousarray(hG[ra]), np.ascontiguousarray(B2.T))
    ref_b = oracle.gemm_f64(np.ascontiguousarray(A2[:, rb].T), hG)
    got_a = dgA.to_numpy().reshape(M, K)[ra].astype(np.float64)
    got_b = dgB.to_numpy().reshape(K, N)[rb].astype(np.float64)
    res["backward_tc_3xbf16_6prod"] = {"fwd_ms": round(f_ms, 3), "dA_ms": round(a_ms, 3), "dB_ms": round(b_ms, 3),
                                       "fwd_plus_adjoint_over_fwd": round((f_ms + a_ms + b_ms) / f_ms, 3),
                                       "normwise_err_vs_fp64": {
                                           "dA": float(np.abs(got_a - ref_a).max() / np.abs(ref_a).max()),
                                           "dB": float(np.abs(got_b - ref_b).max() / np.abs(ref_b).max())},
                                       "note": "two contractions of the forward's size: 3x is the flop bound"}
    out["allpairs_8192x4096x8192"] = res
    del dA, dB, dP, A, B, dG, dgA, dgB, hG, A2, B2, ref_a, ref_b, got_a, got_b
    Ml, Kl, Nl = 4096, 256, 4096
    L_ = oracle.normal_f32(Ml * Kl, 10)
    R_ = oracle.normal_f32(Kl * Nl, 11)
    man = S.Program(S.KIND_ALLPAIRS, "float func(float x, float y){ return x+y; }", ["float"] * 3,
                    source2="float func(float x, float y){ return fabs(x-y); }", identity="0")
    dL, dR, dM = S.DeviceArray.from_numpy(L_), S.DeviceArray.from_numpy(R_), S.DeviceArray(Ml * Nl, np.float32)
    ms = timed(S, lambda: man.launch([dL, dR, dM], rows=Ml, cols=Nl, dim=Kl), 5, 2)
    rm = np.arange(0, Ml, Ml // 16)
    ref_m = oracle.manhattan_f64(np.ascontiguousarray(L_.reshape(Ml, Kl)[rm]), R_.reshape(Kl, Nl))
    got_m = dM.to_numpy().reshape(Ml, Nl)[rm].astype(np.float64)
    man_err = float(np.abs(got_m - ref_m).max() / np.abs(ref_m).max())
    # the same distances through the generic form (user function over row and
    # column accessors, reference AllPairsKernel2.cl): one output per thread
    gen = S.Program(S.KIND_ALLPAIRS_GENERIC,
                    "float func(lmatrix_t* row, rmatrix_t* col, const unsigned int dim) { float s = 0.0f;"
                    " for (unsigned int i = 0; i < dim; ++i) s += fabs(getElementFromRow(row, i) -"
                    " getElementFromColumn(col, i)); return s; }", ["float"] * 3)
    gms = timed(S, lambda: gen.launch([dL, dR, dM], rows=Ml, cols=Nl, dim=Kl), 5, 2)
    got_g = dM.to_numpy().reshape(Ml, Nl)[rm].astype(np.float64)
    out["segmented_10000_vectors"] = segmented(S, oracle, hbm_peak)
    out["segmented_1e6_short_vectors"] = segmented_short(S, oracle, hbm_peak)
    out["manhattan_4096x256x4096"] = {"ms": round(ms, 3),
                                       "Gpairops": round(Ml * Nl * Kl / ms / 1e6, 1),
                                       "TFLOPs_3flop": round(3 * Ml * Nl * Kl / ms / 1e9, 2),
                                       "fp32_frac": round(3 * Ml * Nl * Kl / ms / 1e9 / fp32_peak, 3),
                                       "normwise_err_vs_fp64": man_err,
                                       "generic_form": {
                                           "ms": round(gms, 3),
                                           "TFLOPs_3flop": round(3 * Ml * Nl * Kl / gms / 1e9, 2),
                                           "normwise_err_vs_fp64": float(np.abs(got_g - ref_m).max() /
                                                                         np.abs(ref_m).max())}}
    return out


def segmented_short(S, oracle, hbm_peak):
    """10^6 float32 vectors of 1..199 elements (uniform, seed 1; about 10^8
    elements): inclusive Scan(+) and Reduce(+) per vector, one warp each, against
    the same launches on the flat vector; the per-vector sums checked against
    FP64 on a sample."""
    nseg = 1_000_000
    rng = np.random.default_rng(1)
    lens = rng.integers(1, 200, nseg).astype(np.uint64)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    n = int(off[-1])
    x = oracle.uniform_f32(n, 2, -1.0, 1.0)
    sp = S.Program(S.KIND_SCAN, "float func(float x, float y){ return x+y; }", ["float"], identity="0")
    rp = S.Program(S.KIND_REDUCE, "float func(float x, float y){ return x+y; }", ["float"], identity="0")
    dx, dy, dr, doff = (S.DeviceArray.from_numpy(x), S.DeviceArray(n, np.float32),
                        S.DeviceArray(nseg, np.float32), S.DeviceArray.from_numpy(off))
    plan = S.SegPlan(doff, n)
    # with the plan (one launch per skeleton call), then without it (the
    # offsets pre-pass and separate short / tiled launches on every call)
    seg_scan = timed(S, lambda: sp.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE, segments=plan), 10, 3)
    seg_red = timed(S, lambda: rp.launch([dx, dr], n=n, segments=plan), 10, 3)
    np_scan = timed(S, lambda: sp.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE, segments=doff), 10, 3)
    np_red = timed(S, lambda: rp.launch([dx, dr], n=n, segments=doff), 10, 3)
    rp.launch([dx, dr], n=n, segments=plan)
    sums = dr.to_numpy().astype(np.float64)
    pick = np.arange(0, nseg, nseg // 1000)
    ref = np.array([oracle.sum_f64(x[int(off[i]):int(off[i + 1])]) for i in pick])
    flat_scan = timed(S, lambda: sp.launch([dx, dy], n=n, flags=S.SHAPE_INCLUSIVE), 10, 3)
    flat_red = timed(S, lambda: rp.launch([dx, dr], n=n), 10, 3)
    # the adjoint of the segmented Reduce: each vector's gradient broadcast
    # over its elements, against the flat broadcast of one value
    L = S.lib()
    seg_bc = timed(S, lambda: S.check(L.scl_adjoint_broadcast_segments(dr.ptr, dy.ptr, doff.ptr, nseg, n,
                                                                       S.DTYPE_F32, 0)), 10, 3)
    flat_bc = timed(S, lambda: S.check(L.scl_adjoint_broadcast(dr.ptr, dy.ptr, n, S.DTYPE_F32, 0)), 10, 3)
    S.check(L.scl_adjoint_broadcast_segments(dr.ptr, dy.ptr, doff.ptr, nseg, n, S.DTYPE_F32, 0))
    gb = dy.to_numpy()
    ids = np.repeat(np.arange(nseg), lens.astype(np.int64))
    bc_ok = bool(np.array_equal(gb, dr.to_numpy()[ids]))
    plan.release()
    return {"n_vectors": nseg, "elements": n,
            "scan": {"ms": round(seg_scan, 4), "GBps": round(8 * n / seg_scan / 1e6, 1),
                     "flat_ms": round(flat_scan, 4), "without_plan_ms": round(np_scan, 4)},
            "reduce": {"ms": round(seg_red, 4), "GBps": round(4 * n / seg_red / 1e6, 1),
                       "flat_ms": round(flat_red, 4), "without_plan_ms": round(np_red, 4),
                       "max_abs_err_vs_fp64_sampled": float(np.abs(sums[pick] - ref).max())},
            "broadcast_adjoint": {"ms": round(seg_bc, 4), "GBps": round(4 * n / seg_bc / 1e6, 1),
                                  "flat_ms": round(flat_bc, 4), "exact": bc_ok},
            "note": "with a segment plan: one launch per call, the short vectors' window records "
                    "bulk-copied into shared memory, a thread per vector of up to 256 elements; without "
                    "it the offsets pre-pass runs on every call and each short vector takes a warp"}


def segmented(S, oracle, hbm_peak):
    """10,000 float32 vectors, lengths floor(2^U[6,20]) (seed 12), values
    U[-1,1] (seed 13), back to back: Map(x*x+1) -> inclusive Scan(+) ->
    Reduce(+) per vector, and the adjoints (segmented broadcast, segmented
    reverse scan, Map's vector-Jacobian product).  One launch per skeleton
    for all vectors (a segment plan: the offsets pre-pass ran once, before),
    replayed from a CUDA graph;
    against the same pipeline on one flat vector of the same length and
    against one launch per vector per skeleton (also replayed from a graph,
    so host overhead is not counted)."""
    import ctypes
    L = S.lib()
    nseg = 10_000
    lens = np.floor(2.0 ** oracle.uniform_f32(nseg, 12, 6.0, 20.0).astype(np.float64)).astype(np.uint64)
    off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
    n = int(off[-1])
    x = oracle.uniform_f32(n, 13, -1.0, 1.0)
    FADD = "float func(float x, float y){ return x + y; }"
    mp = S.Program(S.KIND_MAP, "float func(float x){ return x*x + 1.0f; }", ["float", "float"])
    ma = S.Program(S.KIND_MAP_ADJOINT, "float d(float x, float g){ return 2.0f*x*g; }", ["float", "float"], func="d")
    sp = S.Program(S.KIND_SCAN, FADD, ["float"], identity="0")
    rp = S.Program(S.KIND_REDUCE, FADD, ["float"], identity="0")
    dx = S.DeviceArray.from_numpy(x)
    dm, ds = S.DeviceArray(n, np.float32), S.DeviceArray(n, np.float32)
    dgs, dgm, dgx = S.DeviceArray(n, np.float32), S.DeviceArray(n, np.float32), S.DeviceArray(n, np.float32)
    doff = S.DeviceArray.from_numpy(off)
    dr = S.DeviceArray(nseg, np.float32)
    dseed = S.DeviceArray.from_numpy(np.ones(nseg, np.float32))
    flat = S.DeviceArray.from_numpy(np.array([0, n], np.uint64))
    plan, flat_plan = S.SegPlan(doff, n), S.SegPlan(flat, n)

    def fwd(segs, out):
        mp.launch([dx, dm], n=n)
        sp.launch([dm, ds], n=n, flags=S.SHAPE_INCLUSIVE, segments=segs)
        rp.launch([ds, out], n=n, segments=segs)

    def adj(segs, nsegs):
        offs = segs.offsets if isinstance(segs, S.SegPlan) else segs
        S.check(L.scl_adjoint_broadcast_segments(dseed.ptr, dgs.ptr, offs.ptr, nsegs, n, S.DTYPE_F32, 0))
        sp.launch([dgs, dgm], n=n, flags=S.SHAPE_INCLUSIVE | S.SHAPE_REVERSE, segments=segs)
        ma.launch([dx, dgm, dgx], n=n)

    def graph_of(fn):
        fn()  # sizes the workspaces outside the capture
        S.sync()
        S.check(L.scl_graph_begin())
        fn()
        g = ctypes.c_void_p()
        S.check(L.scl_graph_end(ctypes.byref(g)))
        return g

    def time_graph(g, reps):
        return timed(S, lambda: S.check(L.scl_graph_launch(g)), reps, 2)

    res = {"n_vectors": nseg, "elements": n, "mean_length": round(n / nseg, 1),
           "bytes_per_elem_fwd_adjoint": [20, 24]}
    g_fwd = graph_of(lambda: fwd(plan, dr))
    g_adj = graph_of(lambda: adj(plan, nseg))
    dr1 = S.DeviceArray(1, np.float32)
    g_flat_fwd = graph_of(lambda: fwd(flat_plan, dr1))
    g_flat_adj = graph_of(lambda: adj(flat_plan, 1))
    g_np_fwd = graph_of(lambda: fwd(doff, dr))  # without the plan: the pre-pass on every call
    f_ms, a_ms = time_graph(g_fwd, 10), time_graph(g_adj, 10)
    ff_ms, fa_ms = time_graph(g_flat_fwd, 10), time_graph(g_flat_adj, 10)
    np_ms = time_graph(g_np_fwd, 10)
    res["segmented"] = {"fwd_ms": round(f_ms, 3), "adjoint_ms": round(a_ms, 3),
                        "fwd_GBps": round(20 * n / f_ms / 1e6, 1), "adjoint_GBps": round(24 * n / a_ms / 1e6, 1),
                        "fwd_frac": round(20 * n / f_ms / 1e6 / hbm_peak, 3),
                        "fwd_plus_adjoint_over_fwd": round((f_ms + a_ms) / f_ms, 3),
                        "fwd_ms_without_plan": round(np_ms, 3)}
    res["single_flat_vector"] = {"fwd_ms": round(ff_ms, 3), "adjoint_ms": round(fa_ms, 3),
                                 "fwd_GBps": round(20 * n / ff_ms / 1e6, 1),
                                 "adjoint_GBps": round(24 * n / fa_ms / 1e6, 1)}
    res["segmented_over_single_bandwidth"] = {"fwd": round(ff_ms / f_ms, 3), "adjoint": round(fa_ms / a_ms, 3)}
    # correctness on a sample of vectors (FP64)
    fwd(plan, dr)
    got = dr.to_numpy()
    chk = np.arange(0, nseg, 97)
    err = 0.0
    for s_ in chk:
        a, b = int(off[s_]), int(off[s_ + 1])
        v = np.cumsum(x[a:b].astype(np.float64) ** 2 + 1.0).sum()
        err = max(err, abs(float(got[s_]) - v) / abs(v))
    res["max_rel_err_vs_fp64_sampled"] = err
    for g in (g_fwd, g_adj, g_flat_fwd, g_flat_adj, g_np_fwd):
        L.scl_graph_destroy(g)
    # one launch per vector per skeleton, from a graph (forward only)
    views = [(dx.view(int(off[i]), int(lens[i])), dm.view(int(off[i]), int(lens[i])),
              ds.view(int(off[i]), int(lens[i])), dr.view(i, 1), int(lens[i])) for i in range(nseg)]

    def per_vector():
        for vx, vm, vs, vr, ln in views:
            mp.launch([vx, vm], n=ln)
            sp.launch([vm, vs], n=ln, flags=S.SHAPE_INCLUSIVE)
            rp.launch([vs, vr], n=ln)

    g_pv = graph_of(per_vector)
    pv_ms = time_graph(g_pv, 2)
    L.scl_graph_destroy(g_pv)
    res["per_vector_launches"] = {"launches": 3 * nseg, "fwd_ms": round(pv_ms, 3),
                                  "fwd_GBps": round(20 * n / pv_ms / 1e6, 1),
                                  "segmented_speedup": round(pv_ms / f_ms, 2)}
    return res


def run_reference(args):
    """CPU restatement of the same workload on the host cores (the reference
    itself cannot run here: it needs an OpenCL platform and libclang)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import oracle
    n = N_SCAN  # the whole 2^28 workload every step (about 60-70 ms on 16 host cores)
    x = oracle.mod_i32(n, 0, 1001)
    out = np.empty_like(x)
    nt = oracle.threads()
    for _ in range(args.warmup):
        oracle.scan_incl_mod_i32_mt(x, MOD, nt, out)
    t = time.perf_counter()
    for _ in range(args.steps):
        oracle.scan_incl_mod_i32_mt(x, MOD, nt, out)
    sec = (time.perf_counter() - t) / args.steps
    val = 16 * n / sec / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": round(val, 3), "unit": "GB/s",
            "n_gpus": int(os.environ.get("WORLD_SIZE", "1")), "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(sec * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int32", "data": "synthetic (SplitMix64 seed 0, uniform {0..1000})",
            "config": {"workload": WORKLOAD, "n": n, "l2": "inputs (1 GiB) larger than L2; no flush",
                       "parallelism": "single host"},
            "cpu_baseline": {"value": round(val, 3), "unit": "GB/s", "cores": nt, "kind": "port",
                             "sample": "2^28 int32 (the whole workload) per step, scan+mod fused "
                                       "(two-pass chunked)"},
            "e2e": {"value": round(val, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "SkelCL itself needs an OpenCL platform + libclang (absent); this is the oracle port"}
    print(json.dumps(line), flush=True)


CASES = ("scan_int32", "map_mod", "zip_mul", "reduce_f32", "scan_f32", "mapoverlap", "allpairs_simt",
         "allpairs_tc", "manhattan", "segmented_short", "fp32_peak")


def run_case(args):
    """One skeleton kernel, `steps` launches after `warmup`: the small cases
    the ncu summaries under profiles/ were captured on."""
    import oracle
    import skelcl_gb300 as S
    S.init(0)
    n = args.n
    c = args.case
    if c == "fp32_peak":
        peak, res = fp32_peak_measured(S)
        print(json.dumps({"case": c, "rate": peak, "unit": "TFLOP/s", "detail": res,
                          "launches": S.launch_count()}), flush=True)
        return
    if c in ("scan_int32", "map_mod"):
        x = S.DeviceArray.from_numpy(oracle.mod_i32(n, 0, 1001))
        y = S.DeviceArray(n, np.int32)
        if c == "scan_int32":
            p = S.Program(S.KIND_SCAN, "int func(int x, int y){ return x+y; }", ["int"], identity="0")
            fn = lambda: p.launch([x, y], n=n, flags=S.SHAPE_INCLUSIVE)
        else:
            p = S.Program(S.KIND_MAP, "int func(int x){ return x % 7919; }", ["int", "int"])
            fn = lambda: p.launch([x, y], n=n)
        nbytes = 8 * n
    elif c == "segmented_short":
        # n vectors of 1..199 float elements (uniform, seed 1), values
        # U[-1,1] (seed 2): a segmented inclusive Scan(+) and Reduce(+) per
        # step, and the Reduce's adjoint (each vector's value broadcast)
        rng = np.random.default_rng(1)
        lens = rng.integers(1, 200, n).astype(np.uint64)
        off = np.concatenate([[0], np.cumsum(lens)]).astype(np.uint64)
        ne = int(off[-1])
        a = S.DeviceArray.from_numpy(oracle.uniform_f32(ne, 2, -1.0, 1.0))
        z, r, doff = S.DeviceArray(ne, np.float32), S.DeviceArray(n, np.float32), S.DeviceArray.from_numpy(off)
        sp = S.Program(S.KIND_SCAN, "float func(float x, float y){ return x+y; }", ["float"], identity="0")
        rp = S.Program(S.KIND_REDUCE, "float func(float x, float y){ return x+y; }", ["float"], identity="0")

        plan = S.SegPlan(doff, ne)

        L = S.lib()

        def fn():
            sp.launch([a, z], n=ne, flags=S.SHAPE_INCLUSIVE, segments=plan)
            rp.launch([a, r], n=ne, segments=plan)
            S.check(L.scl_adjoint_broadcast_segments(r.ptr, z.ptr, doff.ptr, n, ne, S.DTYPE_F32, 0))
        nbytes = 16 * ne
    elif c in ("zip_mul", "reduce_f32", "scan_f32"):
        a = S.DeviceArray.from_numpy(oracle.uniform_f32(n, 0, -1.0, 1.0))
        b = S.DeviceArray.from_numpy(oracle.uniform_f32(n, 1, -1.0, 1.0))
        z = S.DeviceArray(n, np.float32)
        if c == "zip_mul":
            p = S.Program(S.KIND_ZIP, "float func(float x, float y){ return x*y; }", ["float"] * 3)
            fn = lambda: p.launch([a, b, z], n=n)
            nbytes = 12 * n
        elif c == "reduce_f32":
            p = S.Program(S.KIND_REDUCE, "float func(float x, float y){ return x+y; }", ["float"], identity="0")
            fn = lambda: p.launch([a, z], n=n)
            nbytes = 4 * n
        else:
            p = S.Program(S.KIND_SCAN, "float func(float x, float y){ return x+y; }", ["float"], identity="0.0f")
            fn = lambda: p.launch([a, z], n=n, flags=S.SHAPE_INCLUSIVE)
            nbytes = 8 * n
    elif c == "mapoverlap":
        side = int(round(n ** 0.5))
        img = S.DeviceArray.from_numpy(oracle.uniform_f32(side * side, 5, 0.0, 255.0))
        out = S.DeviceArray(side * side, np.float32)
        w = S.DeviceArray.from_numpy(oracle.gaussian_weights(5, 2.0).ravel())
        src = ("float func(input_matrix_t img, __global float* w) { float s = 0.0f;"
               " for (int dy = -5; dy <= 5; ++dy) for (int dx = -5; dx <= 5; ++dx)"
               "  s += getData(img, dx, dy) * w[(dy + 5) * 11 + (dx + 5)]; return s; }")
        p = S.Program(S.KIND_MAPOVERLAP, src, ["float", "float"], overlap_range=5, padding=S.PAD_NEAREST)
        fn = lambda: p.launch([img, out], rows=side, cols=side, extra=S.buffer(w))
        nbytes = 8 * side * side
    else:
        side = int(round(n ** (1 / 3)))
        K = 256 if c == "manhattan" else side
        A = S.DeviceArray.from_numpy(oracle.normal_f32(side * K, 7))
        B = S.DeviceArray.from_numpy(oracle.normal_f32(K * side, 8))
        P = S.DeviceArray(side * side, np.float32)
        zsrc = "float func(float x, float y){ return fabs(x-y); }" if c == "manhattan" else \
            "float func(float x, float y){ return x*y; }"
        p = S.Program(S.KIND_ALLPAIRS, "float func(float x, float y){ return x+y; }", ["float"] * 3,
                      source2=zsrc, identity="0")
        var = S.VARIANT_TC3XBF16 if c == "allpairs_tc" else S.VARIANT_SIMT
        fn = lambda: p.launch([A, B, P], rows=side, cols=side, dim=K, tuning=S.Tuning(variant=var))
        nbytes = 2 * side * side * K  # flop
    ms = timed(S, fn, args.steps, args.warmup)
    print(json.dumps({"case": c, "n": n, "ms": round(ms, 4),
                      "rate": round(nbytes / ms / 1e6, 1),
                      "unit": "GFLOP/s" if c.startswith(("allpairs", "manhattan")) else "GB/s",
                      "launches": S.launch_count()}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--headline-only", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--case", choices=CASES, help="time one skeleton kernel (profiling)")
    ap.add_argument("--n", type=int, default=1 << 26,
                    help="--case size (elements; segmented_short: vectors)")
    args = ap.parse_args()
    if args.warmup < 1:
        args.warmup = 1
    if args.case:
        run_case(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
