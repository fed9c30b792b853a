"""Benchmark: histories/s and dose efficiency 1/(sigma^2 T) of the GB300
transport engine on the heterogeneous slab phantom (64^3 x 0.25 cm, water /
lung / bone / water, 10x10 cm photon field with a 0.1-6 MeV bremsstrahlung-like
spectrum), one batch of 1e7 histories per step.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Prints one JSON line.  A step is one statistical batch of histories transported
to completion; inputs (phantom, tables) are resident on the device for
`value`; `e2e` repeats the step through the C ABI with host buffers (phantom
upload and tally read-back inside the timed region).  Under torchrun every
rank transports its own history range (weak scaling, no collective on the
data path).  `--impl reference` times the CPU implementation of the same
transport (the FP64 restatement of EGSnrc's PHOTON/ELECTR loop) on the host
cores instead.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

ALG_BYTES_PER_STEP = 104      # particle record read + write (48 + 48) + one FP64 tally update
ALG_BYTES_PER_PUSH = 48       # one secondary record written to a queue


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="slab64")
    ap.add_argument("--histories", type=float, default=1e8,
                    help="histories per step (one batch); the default is the slab64 configuration's 1e8")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-phantoms leg of the default bench")
    ap.add_argument("--precision", type=int, default=32)
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison leg")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--capacity", type=int, default=0, help="particle-queue capacity (0 = engine default)")
    ap.add_argument("--chunk", type=int, default=0, help="histories per wavefront chunk (0 = automatic)")
    ap.add_argument("--block-size", type=int, default=0, help="threads per CTA of the transport kernels (0 = engine)")
    ap.add_argument("--graph", type=int, default=0, choices=[0, 1, 2],
                    help="wavefront rounds: 0 direct launches, 1 graph replay, 2 device-side loop per chunk")
    ap.add_argument("--ctas-per-sm", type=int, default=0, help="resident CTAs per SM (0 = as many as fit)")
    ap.add_argument("--inter-batch", type=int, default=0,
                    help="lanes a warp gathers before it samples their interactions together (0 = engine default)")
    ap.add_argument("--clock-period", type=float, default=0.2, help="seconds between clock samples")
    ap.add_argument("--clock-mode", default="nvml", choices=["nvml", "process", "off"])
    ap.add_argument("--adjoint", action="store_true",
                    help="also time the seed-replay gradient of sum (D - T)^2 over all voxel densities "
                         "(T from a second density map; the perturbed64 workload is config c5)")
    ap.add_argument("--howfarless", action="store_true",
                    help="DOSXYZnrc HOWFARLESS transport (homogeneous phantoms: water30, water128e)")
    ap.add_argument("--scale", type=float, default=0.005,
                    help="batched64: fraction of each phantom's 1e6-5e7 histories run per step")
    return ap.parse_args()


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        if args.impl == "ours":
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
        return ws, rank, local, dist
    return 1, 0, 0, None


class ClockSampler:
    """SM clocks and clock-event (throttle) reasons sampled during the timed
    region through NVML in-process (libnvidia-ml via ctypes; read-only
    queries), falling back to nvidia-smi once per second."""

    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, index=0, period=0.2, mode="nvml"):
        self.index = index
        self.period = period
        self.mode = mode
        self._proc = None
        self.samples = []     # (sm_mhz, max_mhz, reasons_bitmask, power_w)
        self._stop = threading.Event()
        self._t = None
        self._nvml = None
        if mode != "nvml":
            return
        try:
            import ctypes
            L = ctypes.CDLL("libnvidia-ml.so.1")
            if L.nvmlInit_v2() == 0:
                h = ctypes.c_void_p()
                if L.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(index), ctypes.byref(h)) == 0:
                    self._nvml = (ctypes, L, h)
        except Exception:
            self._nvml = None

    def _sample_nvml(self):
        ctypes, L, h = self._nvml
        clk, mx, pw = ctypes.c_uint(0), ctypes.c_uint(0), ctypes.c_uint(0)
        rs = ctypes.c_ulonglong(0)
        L.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk))          # NVML_CLOCK_SM
        L.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))
        L.nvmlDeviceGetPowerUsage(h, ctypes.byref(pw))
        L.nvmlDeviceGetCurrentClocksThrottleReasons(h, ctypes.byref(rs))
        self.samples.append((float(clk.value), float(mx.value), int(rs.value), pw.value / 1e3))

    def _sample_smi(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                              "--format=csv,noheader,nounits"], stdout=subprocess.PIPE,
                             stderr=subprocess.DEVNULL, text=True, timeout=5).stdout.strip()
        f = [x.strip() for x in out.split(",")]
        bits = 0
        for b, v in zip((0x8, 0x40, 0x20, 0x4), f[3:7]):
            if v.lower() == "active":
                bits |= b
        self.samples.append((float(f[0]), float(f[1]), bits, float(f[2]) if f[2][:1].isdigit() else 0.0))

    def _run(self):
        while not self._stop.is_set():
            try:
                if self._nvml:
                    self._sample_nvml()
                else:
                    self._sample_smi()
            except Exception:
                pass
            self._stop.wait(self.period if self._nvml else 1.0)

    def __enter__(self):
        if self.mode == "off":
            return self
        if self.mode == "process":   # nvidia-smi sampling in its own process
            self._proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,"
                 "clocks_event_reasons.active,power.draw", "--format=csv,noheader,nounits",
                 "-lms", str(int(1000 * self.period))], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            return self
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        if self._proc is not None:
            self._proc.terminate()
            out, _ = self._proc.communicate(timeout=10)
            for line in out.splitlines():
                f = [x.strip() for x in line.split(",")]
                try:
                    self.samples.append((float(f[0]), float(f[1]), int(f[2], 16), float(f[3])))
                except (ValueError, IndexError):
                    pass
            return
        if self._t is not None:
            self._stop.set()
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [s[0] for s in self.samples]
        reasons = sorted({name for s in self.samples for bit, name in self.REASONS.items() if s[2] & bit})
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(s[1] for s in self.samples),
                "reasons": reasons, "samples": len(self.samples),
                "power_w_max": max(s[3] for s in self.samples),
                "source": self.mode if self.mode != "nvml" else ("nvml" if self._nvml else "nvidia-smi")}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel, workload, steps_per_launch):
    """DRAM bytes (read + write) per launch of `kernel`, from the committed ncu
    capture of a smaller case of the same workload (profiles/ncu_traffic.json:
    measured DRAM bytes per transport step), scaled to this run's transport
    steps per launch; None without a capture of this kernel and workload."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return d[workload][kernel]["dram_bytes_per_step"] * steps_per_launch
    except Exception:
        return None


def pinned_pair(n):
    """Two float64 host arrays of n elements in page-locked memory: the
    e2e legs read the tallies into these every step."""
    import torch
    return tuple(torch.empty(n, dtype=torch.float64, pin_memory=True).numpy() for _ in range(2))


def sigma_eff(sum_, sum2, nb, frac=0.5):
    m = sum_ / nb
    var = np.maximum(sum2 / nb - m * m, 0) / max(nb - 1, 1)
    dose = sum_
    sel = dose > frac * dose.max()
    rel = np.sqrt(var[sel]) * nb / np.maximum(sum_[sel], 1e-300)
    return float(np.sqrt(np.mean(rel * rel))), int(sel.sum())


def cpu_sample(wl, seconds, threads, seed):
    """Times the CPU oracle on a bounded sample of the workload (rank 0, N = 1)."""
    from oracle.oracle_binding import Oracle
    ora = Oracle(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], fast=True)
    ora.set_geometry(wl["geometry"])
    ora.set_source(wl["source"])
    n0 = 400 * threads
    t0 = time.perf_counter()
    ora.run(n0, nbatch=1, seed=seed, first=0, threads=threads)
    dt0 = time.perf_counter() - t0
    n = max(threads, int(n0 * max(seconds - dt0, 0.5) / max(dt0, 1e-3)))
    t1 = time.perf_counter()
    ora.run(n, nbatch=1, seed=seed, first=n0, threads=threads)
    dt = time.perf_counter() - t1
    return n, dt


def reference_arm(args, wl, ws, rank, dist):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    K, W = args.steps, args.warmup
    # size one step to about 4 s of host work
    from oracle.oracle_binding import Oracle
    ora = Oracle(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], fast=True)
    ora.set_geometry(wl["geometry"])
    ora.set_source(wl["source"])
    n0 = 200 * threads
    t0 = time.perf_counter()
    ora.run(n0, nbatch=1, seed=wl["seed"], first=0, threads=threads)
    rate = n0 / max(time.perf_counter() - t0, 1e-3)
    per_step = max(threads, int(rate * 4.0))
    first = n0
    for _ in range(W):
        ora.run(per_step, nbatch=1, seed=wl["seed"], first=first, threads=threads)
        first += per_step
    ora2 = Oracle(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], fast=True)
    ora2.set_geometry(wl["geometry"])
    ora2.set_source(wl["source"])
    t0 = time.perf_counter()
    for _ in range(K):
        ora2.run(per_step, nbatch=1, seed=wl["seed"], first=first, threads=threads)
        first += per_step
    T = time.perf_counter() - t0
    value = per_step * K / T
    s, s2, tot = ora2.tallies()
    sig, nsel = sigma_eff(s, s2, K) if K > 1 else (None, 0)
    eff = (1.0 / (sig * sig * T)) if sig else None
    line = {"impl": "reference", "metric": "histories_per_second", "value": value, "unit": "histories/s",
            "n_gpus": args.gpus, "steps": K, "warmup": W, "ms_per_step": 1e3 * T / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": config_of(wl), "histories_per_step": int(per_step),
            "dose_efficiency": eff, "sigma_bar_50pct": sig,
            "cpu_baseline": {"value": value, "unit": "histories/s", "cores": threads, "kind": "port",
                             "sample": "%d histories per step x %d steps of %s (FP64 CPU restatement of the "
                                       "reference transport, -O3 -ffast-math, one thread per core)"
                                       % (per_step, K, wl["name"])},
            "e2e": {"value": value, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def config_of(wl, howfarless=False):
    """The workload: the same dict for both arms.  How many histories one
    step transports is a measurement parameter, reported beside it
    (`histories_per_step`): the rate is per history."""
    g = wl["geometry"]
    return {"workload": wl["name"] + ("-howfarless" if howfarless else ""),
            "phantom": "%dx%dx%d voxels" % (g.nx, g.ny, g.nz),
            "media": wl["media"], "batches_per_step": 1,
            "ecut_MeV": wl["ecut"], "pcut_MeV": wl["pcut"],
            "l2": "256 MiB buffer written between timed steps"}


def batched_sigma(eng, probs, nb):
    """Mean squared relative 1-sigma over the voxels above half of each
    phantom's own maximum, over all phantoms (nb batches)."""
    s_all, s2_all, _ = eng.tallies()
    rel2, n = [], 0
    for k in range(len(probs)):
        off, nv, _ = eng.phantom_info(k)
        s, s2 = s_all[off:off + nv], s2_all[off:off + nv]
        if s.max() <= 0:
            continue
        m = s / nb
        var = np.maximum(s2 / nb - m * m, 0) / max(nb - 1, 1)
        sel = s > 0.5 * s.max()
        rel2.append(var[sel] * nb * nb / (s[sel] * s[sel]))
        n += int(sel.sum())
    r = np.concatenate(rel2)
    return float(np.sqrt(np.mean(r))), n


def batched_oracle(wl, frac, threads, first):
    """CPU oracle over every phantom of the batched workload, `frac` of each
    phantom's step histories; returns (histories, seconds)."""
    from oracle.oracle_binding import Oracle
    ora = Oracle(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], fast=True)
    n, t = 0, 0.0
    for p in wl["problems"]:
        m = max(threads, int(p["histories"] * frac))
        ora.set_geometry(p["geometry"])
        ora.set_source(p["source"])
        t0 = time.perf_counter()
        ora.run(m, nbatch=1, seed=p["seed"], first=first, threads=threads)
        t += time.perf_counter() - t0
        n += m
    return n, t


def batched_config(wl, args):
    ps = wl["problems"]
    return {"workload": "batched64", "phantoms": len(ps), "edges_voxels": [int(p["edge"]) for p in ps][:64],
            "voxel_cm": 0.2, "media": wl["media"], "histories_per_step": int(sum(p["histories"] for p in ps)),
            "history_scale": args.scale, "batches_per_step": 1, "ecut_MeV": wl["ecut"], "pcut_MeV": wl["pcut"],
            "l2": "256 MiB buffer written between timed steps"}


def bench_batched(args, ws, rank, local, dist):
    """Many phantoms per step (one egsgpu_run_phantoms call) against the same
    phantoms run one after another; prints the line."""
    line = batched_measure(args, ws, rank, local, dist, args.steps, args.warmup, args.no_cpu, 0.25)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)


def batched_measure(args, ws, rank, local, dist, K, Wm, no_cpu, fp64_frac):
    """The batched64 workload: K timed steps, each one egsgpu_run_phantoms
    call over all 64 phantoms; returns the JSON line (rank 0) or None."""
    from egsnrc_gb300 import workloads as W
    wl = W.batched64(scale=args.scale)
    ps = wl["problems"]
    for p in ps:          # every rank transports its own histories (weak scaling)
        p["seed"] += 7919 * rank
    H = sum(p["histories"] for p in ps)
    threads = os.cpu_count() or 1
    if args.impl == "reference":
        if rank != 0:
            return None
        n0, t0 = batched_oracle(wl, 2e-3, threads, 0)
        frac = 2e-3 * 4.0 / max(t0, 1e-3)          # about 4 s of host work per step
        for _ in range(Wm):
            batched_oracle(wl, frac, threads, 10 ** 7)
        n, T = 0, 0.0
        for _ in range(K):
            a, b = batched_oracle(wl, frac, threads, 2 * 10 ** 7)
            n += a; T += b
        value = n / T
        line = {"impl": "reference", "metric": "histories_per_second", "value": value, "unit": "histories/s",
                "n_gpus": args.gpus, "steps": K, "warmup": Wm, "ms_per_step": 1e3 * T / K,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": batched_config(wl, args),
                "cpu_baseline": {"value": value, "unit": "histories/s", "cores": threads, "kind": "port",
                                 "sample": "%.2g of every phantom's step histories per step x %d steps (FP64 CPU "
                                           "restatement, one thread per core)" % (frac, K)},
                "e2e": {"value": value, "unit": "histories/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        return line
    import torch
    import egsnrc_gb300 as eg
    torch.cuda.set_device(local)
    ekw = dict(capacity=args.capacity, chunk=args.chunk, block_size=args.block_size, ctas_per_sm=args.ctas_per_sm,
               use_graph=args.graph, inter_batch=args.inter_batch)
    eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=args.precision, **ekw)
    eng.set_phantoms(ps)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    flush.zero_()
    torch.cuda.synchronize()
    for _ in range(Wm):
        eng.run_phantoms(nbatch=1)
    eng.reset()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local, args.clock_period, args.clock_mode) as clk:
        torch.cuda.synchronize()
        start.record()
        for _ in range(K):
            flush.zero_()
            eng.run_phantoms(nbatch=1)
        stop.record()
        torch.cuda.synchronize()
    T = start.elapsed_time(stop) / 1e3
    if dist:
        tt = torch.tensor([T], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        T = float(tt.item())
    prof = eng.profile()
    sig, nsel = batched_sigma(eng, ps, K) if K > 1 else (None, 0)
    value = H * ws * K / T
    eff = (1.0 / (sig * sig * T)) if sig else None
    kern = "electron" if prof["ms_electron"] >= prof["ms_photon"] else "photon"
    steps_k, pushes_k = prof[kern + "_steps"], prof[kern + "_pushes"]
    ms_k, n_k = prof["ms_" + kern], max(prof["launches_" + kern], 1)
    bytes_k = steps_k * ALG_BYTES_PER_STEP + pushes_k * ALG_BYTES_PER_PUSH
    achieved = bytes_k / (ms_k / 1e3) / 1e9 if ms_k > 0 else None
    peak, peak_kind = measured_peak_hbm()
    roof = {"bound": "hbm", "kernel": "k_" + kern, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "peak_source": peak_kind,
            "traffic": ncu_traffic("k_" + kern, "batched64", steps_k / n_k), "alg_bytes_per_launch": bytes_k / n_k,
            "launches": n_k, "ms_per_launch": ms_k / n_k, "steps_per_launch": steps_k / n_k,
            "kernel_share": {k: prof["ms_" + k] / max(1e-9, sum(prof["ms_" + j] for j in
                                                                  ("source", "photon", "electron", "batch")))
                             for k in ("source", "photon", "electron", "batch")}}
    launches = sum(prof["launches_" + k] for k in ("source", "photon", "electron", "batch"))
    eng.close()

    # e2e: phantoms uploaded from host arrays, run, tallies read back, every step
    e2e_eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=args.precision, **ekw)
    h2d = sum(p["geometry"].xb.nbytes + p["geometry"].yb.nbytes + p["geometry"].zb.nbytes + p["geometry"].med.nbytes
              + p["geometry"].rhor.nbytes for p in ps)
    nv_all = sum(p["geometry"].nvox for p in ps)
    host_out = pinned_pair(nv_all)   # the caller's tally buffers, pinned and reused every step

    def e2e_step():
        e2e_eng.set_phantoms(ps)
        e2e_eng.run_phantoms(nbatch=1)
        e2e_eng.tallies(out=host_out)
    for _ in range(Wm):   # the same untimed warm-up as the device-timed leg
        e2e_step()
    torch.cuda.synchronize()
    te0 = time.perf_counter()
    for _ in range(K):
        flush.zero_()
        e2e_step()
    torch.cuda.synchronize()
    Te = time.perf_counter() - te0
    e2e_eng.close()
    line = {"metric": "histories_per_second", "value": value, "unit": "histories/s", "n_gpus": ws, "steps": K,
            "warmup": Wm, "ms_per_step": 1e3 * T / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == 32 else "f64", "data": "synthetic",
            "config": batched_config(wl, args), "dose_efficiency": eff, "dose_efficiency_unit": "1/(sigma^2 s)",
            "sigma_bar_50pct": sig, "voxels_above_50pct": nsel,
            "e2e": {"value": H * ws * K / Te, "unit": "histories/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(2 * nv_all * 8 + 64),
                    "path": "egsgpu_set_phantoms + egsgpu_run_phantoms + egsgpu_get_tallies"},
            "roofline": roof, "gpu_launches": int(launches),
            "autotuner": {"chunk": prof["chunk"], "launch_shape": prof["launch_shape"],
                          "shapes": "threads per CTA / CTAs per SM of photon, electron kernels relative to the "
                                    "most that fit: 0 128/0/0, 1 64/0/0, 2 96/0/0, 3 128/0/-1, 4 128/-2/0, 5 64/0/-2"}}
    if rank == 0 and not args.no_fp64:
        # the same phantoms one after another (egsgpu_run per phantom): FP32, and the plain FP64 form
        for prec, key, frac in ((args.precision, "one_at_a_time", 1.0), (64, "fp64_one_at_a_time", fp64_frac)):
            e1 = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=prec, **ekw)
            n1, T1 = 0, 0.0
            rel2 = []
            for p in ps:
                e1.set_geometry(p["geometry"])
                e1.set_source(p["source"])
                m = max(2, int(p["histories"] * frac))
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for k in range(2):
                    e1.run(m, nbatch=1, seed=p["seed"], first=k * m)
                torch.cuda.synchronize()
                T1 += time.perf_counter() - t0
                n1 += 2 * m
                s1, s21, _ = e1.tallies()
                if s1.max() > 0:
                    mm = s1 / 2
                    var = np.maximum(s21 / 2 - mm * mm, 0)
                    sel = s1 > 0.5 * s1.max()
                    rel2.append(var[sel] * 4 / (s1[sel] * s1[sel]))
            e1.close()
            sig1 = float(np.sqrt(np.mean(np.concatenate(rel2))))
            line[key] = {"value": n1 / T1, "unit": "histories/s", "dose_efficiency": 1.0 / (sig1 * sig1 * T1),
                         "histories_fraction": frac}
        if eff:
            line["efficiency_ratio_batched_fp32_over_fp64"] = eff / line["fp64_one_at_a_time"]["dose_efficiency"]
    line["clocks"] = clk.summary()
    if rank == 0 and ws == 1 and not no_cpu:
        n0, t0 = batched_oracle(wl, 1e-3, threads, 10 ** 8)
        frac = 1e-3 * args.cpu_seconds / max(t0, 1e-3)
        n, dt = batched_oracle(wl, frac, threads, 2 * 10 ** 8)
        line["cpu_baseline"] = {"value": n / dt, "unit": "histories/s", "cores": threads, "kind": "port",
                                "sample": "%d histories over all %d phantoms on %d host threads, %.1f s"
                                          % (n, len(ps), threads, dt)}
    return line if rank == 0 else None


def fp32_vs_fp64(wl, eg, ekw, n, seed, nb=10):
    """The FP32 build's error against the FP64 build on the same histories
    (common random numbers), nb batches of n/nb: relative difference of the
    total deposited energy with its standard error from the paired batches,
    and per voxel above 20% of Dmax the paired z = mean difference / its
    standard error (mean z^2 is 1 for an unbiased FP32 build) and the median
    relative difference."""
    per = n // nb
    out = {}
    for prec in (32, 64):
        e = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=prec, **ekw)
        e.set_geometry(wl["geometry"])
        e.set_source(wl["source"])
        prev = np.zeros(wl["geometry"].nvox)
        rows = []
        for b in range(nb):
            e.run(per, nbatch=1, seed=seed, first=b * per)
            s, _, _ = e.tallies()
            rows.append(s - prev)
            prev = s
        out[prec] = np.array(rows)
        wide = e.profile().get("electron_wide_steps", 0.0) if prec == 32 else None
        steps = e.profile()["electron_steps"] if prec == 32 else None
        e.close()
    d = out[32] - out[64]
    ref = out[64].mean(axis=0)
    sel = ref > 0.2 * ref.max()
    md, sd = d.mean(axis=0)[sel], d.std(axis=0, ddof=1)[sel]
    z = np.where(sd > 0, md / np.maximum(sd / np.sqrt(nb), 1e-300), 0.0)
    bt = d.sum(axis=1)
    tot = out[64].sum()
    return {"histories": int(per * nb), "batches": nb, "total_rel": float(bt.sum() / tot),
            "total_rel_sigma": float(bt.std(ddof=1) * np.sqrt(nb) / tot), "voxels": int(sel.sum()),
            "voxel_mean_z2": float(np.mean(z * z)), "voxel_frac_abs_z_lt2": float(np.mean(np.abs(z) < 2)),
            "voxel_median_rel": float(np.median(np.abs(md) / ref[sel])),
            "electron_steps_in_fp64": float(wide / steps) if steps else 0.0}


def simt_roofline(prof):
    """Lane occupancy of the transport kernels' persistent warps, from the
    engine's device counters: mean busy lanes per warp iteration out of 32
    (the ceiling of SIMT efficiency; divergence within the step lowers the
    issued fraction further, see the ncu summaries in profiles/)."""
    out = {}
    for k in ("photon", "electron"):
        b = prof.get(k + "_busy_lanes", 0.0)
        out[k] = {"busy_lanes_per_iteration": b, "frac": b / 32.0,
                  "steps_per_s": prof[k + "_steps"] / (prof["ms_" + k] / 1e3) if prof["ms_" + k] > 0 else None}
    return out


def adjoint_leg(args, wl, eg, ekw, H):
    """Forward run plus egsgpu_adjoint for L = sum (D - T)^2, T simulated on a
    second density map (uniform +-10% perturbations from seed 12)."""
    import torch
    g = wl["geometry"]
    rng = np.random.default_rng(12)
    gt = eg.XYZGeometry(g.xb, g.yb, g.zb, g.med, 1.0 + 0.1 * rng.uniform(-1.0, 1.0, g.nvox))
    e = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=args.precision, **ekw)
    e.set_source(wl["source"])
    e.set_geometry(gt)
    e.run(H, nbatch=10, seed=wl["seed"] + 1)
    T, _ = e.dose()
    e.set_geometry(g)
    e.reset()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e.run(H, nbatch=10, seed=wl["seed"])
    D, _ = e.dose()
    t1 = time.perf_counter()
    grad = e.adjoint(2 * (D - T), H, seed=wl["seed"])
    t2 = time.perf_counter()
    e.close()
    return {"histories": int(H), "forward_s": t1 - t0, "adjoint_s": t2 - t1, "gradient_voxels": int(g.nvox),
            "loss": float(((D - T) ** 2).sum()), "grad_abs_max": float(np.abs(grad).max()),
            "path": "egsgpu_run + egsgpu_get_dose, then egsgpu_adjoint (two replays of the same histories)"}


def main():
    args = parse()
    from egsnrc_gb300 import workloads as W
    ws, rank, local, dist = dist_setup(args)
    if args.workload == "batched64":
        bench_batched(args, ws, rank, local, dist)
        if dist:
            dist.barrier()
            if args.impl != "reference":
                dist.destroy_process_group()
        return
    wl = W.WORKLOADS[args.workload]()
    if args.impl == "reference":
        reference_arm(args, wl, ws, rank, dist)
        if dist:
            dist.barrier()
        return
    import torch
    import egsnrc_gb300 as eg
    torch.cuda.set_device(local)
    H = int(args.histories)
    K, Wm = args.steps, args.warmup
    ekw = dict(capacity=args.capacity, chunk=args.chunk, howfarless=int(args.howfarless), block_size=args.block_size,
               ctas_per_sm=args.ctas_per_sm, use_graph=args.graph, inter_batch=args.inter_batch)
    eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=args.precision, **ekw)
    eng.set_geometry(wl["geometry"])
    eng.set_source(wl["source"])
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    flush.zero_()   # loads torch's fill kernel before anything is timed
    torch.cuda.synchronize()
    # History indices are 32-bit Philox keys: each leg (device-timed, e2e,
    # FP64, FP32-vs-FP64, CPU sample) and each rank draws from its own seed
    # and counts histories from 0, so no leg repeats another's histories.
    seed0 = wl["seed"] + 7919 * rank
    if (K + Wm) * H >= 2 ** 32:
        raise SystemExit("steps x histories per step must stay below 2^32 histories per leg")
    first = 0
    for _ in range(Wm):
        eng.run(H, nbatch=1, seed=seed0, first=first)
        first += H
    eng.reset()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local, args.clock_period, args.clock_mode) as clk:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        start.record()
        for _ in range(K):
            flush.zero_()
            eng.run(H, nbatch=1, seed=seed0, first=first)
            first += H
        stop.record()
        torch.cuda.synchronize()
        t_host = time.perf_counter() - t0
    T = start.elapsed_time(stop) / 1e3
    if dist:
        tt = torch.tensor([T], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        T = float(tt.item())
    prof = eng.profile()
    s, s2, tot = eng.tallies()
    sig, nsel = sigma_eff(s, s2, K) if K > 1 else (None, 0)
    value = H * ws * K / T
    combined = None
    if dist:
        # the ranks' shards of one problem combine into one result
        # (egsgpu_combine_checkpoints, the .egsdat combine)
        blobs = [None] * ws
        dist.all_gather_object(blobs, eng.checkpoint())
        if rank == 0:
            comb = blobs[0]
            for b in blobs[1:]:
                comb = eg.combine_checkpoints(comb, b)
            c = eg.checkpoint_arrays(comb)
            parts = [eg.checkpoint_arrays(b) for b in blobs]
            assert c["histories"] == H * K * ws and c["batches"] == K * ws
            assert abs(c["deposited"] - sum(x["deposited"] for x in parts)) <= 1e-9 * c["deposited"]
            csig, cn = sigma_eff(c["sum"], c["sum2"], c["batches"])
            combined = {"histories": c["histories"], "batches": c["batches"], "sigma_bar_50pct": csig,
                        "voxels_above_50pct": cn, "path": "egsgpu_checkpoint on every rank + egsgpu_combine_checkpoints"}
    eff = (1.0 / (sig * sig * T)) if sig else None

    # roofline of the dominant kernel: algorithmic bytes / CUDA-event kernel time
    kern = "electron" if prof["ms_electron"] >= prof["ms_photon"] else "photon"
    steps_k = prof[kern + "_steps"]
    pushes_k = prof[kern + "_pushes"]
    ms_k, n_k = prof["ms_" + kern], max(prof["launches_" + kern], 1)
    bytes_k = steps_k * ALG_BYTES_PER_STEP + pushes_k * ALG_BYTES_PER_PUSH
    achieved = bytes_k / (ms_k / 1e3) / 1e9 if ms_k > 0 else None
    peak, peak_kind = measured_peak_hbm()
    traffic = ncu_traffic("k_" + kern, wl["name"] + ("-howfarless" if args.howfarless else ""), steps_k / n_k)
    roof = {"bound": "hbm", "kernel": "k_" + kern, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None, "peak_source": peak_kind,
            "traffic": traffic, "alg_bytes_per_launch": bytes_k / n_k, "launches": n_k,
            "ms_per_launch": ms_k / n_k, "steps_per_s": steps_k / (ms_k / 1e3) if ms_k > 0 else None,
            "steps_per_launch": steps_k / n_k, "pushes_per_launch": pushes_k / n_k,
            "launches_photon": prof["launches_photon"], "launches_electron": prof["launches_electron"],
            "steps_photon": prof["photon_steps"], "steps_electron": prof["electron_steps"],
            "kernel_share": {k: prof["ms_" + k] / max(1e-9, sum(prof["ms_" + j] for j in
                                                                  ("source", "photon", "electron", "batch")))
                             for k in ("source", "photon", "electron", "batch")}}
    launches = sum(prof["launches_" + k] for k in ("source", "photon", "electron", "batch"))

    # e2e through the C ABI with host buffers: phantom upload + run + tally read-back
    g = wl["geometry"]
    e2e_eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=args.precision, **ekw)
    e2e_eng.set_geometry(g)
    e2e_eng.set_source(wl["source"])
    h2d = g.xb.nbytes + g.yb.nbytes + g.zb.nbytes + g.med.nbytes + g.rhor.nbytes
    d2h = 2 * g.nvox * 8 + 8 * 8

    host_out = pinned_pair(g.nvox)   # the caller's tally buffers, pinned and reused every step

    first = 0

    def e2e_step(first):
        e2e_eng.set_geometry(g)
        e2e_eng.run(H, nbatch=1, seed=seed0 + 1000, first=first)
        return e2e_eng.tallies(out=host_out)
    for _ in range(Wm):   # the same untimed warm-up as the device-timed leg
        e2e_step(first)
        first += H
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    te0 = time.perf_counter()
    for _ in range(K):
        flush.zero_()
        ss, ss2, _ = e2e_step(first)
        first += H
    torch.cuda.synchronize()
    Te = time.perf_counter() - te0
    if dist:
        tt = torch.tensor([Te], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        Te = float(tt.item())
    e2e = {"value": H * ws * K / Te, "unit": "histories/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "path": "egsgpu_set_xyz_geometry + egsgpu_run + egsgpu_get_tallies"}

    line = {"metric": "histories_per_second", "value": value, "unit": "histories/s", "n_gpus": ws, "steps": K,
            "warmup": Wm, "ms_per_step": 1e3 * T / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if args.precision == 32 else "f64", "data": "synthetic",
            "config": config_of(wl, args.howfarless), "histories_per_step": int(H), "dose_efficiency": eff,
            "dose_efficiency_unit": "1/(sigma^2 s)",
            "sigma_bar_50pct": sig, "voxels_above_50pct": nsel, "e2e": e2e, "roofline": roof,
            "gpu_launches": int(launches), "host_seconds": t_host,
            "autotuner": {"chunk": prof["chunk"], "launch_shape": prof["launch_shape"]}}
    if combined:
        line["combined"] = combined

    if rank == 0 and args.adjoint:
        line["adjoint"] = adjoint_leg(args, wl, eg, ekw, H)
    if rank == 0 and not args.no_fp64 and args.precision == 32:
        # the plain FP64 GPU form on the same problem, timed the same way
        # (CUDA events on the launching stream around 2 steps of H/10)
        H64 = max(H // 10, 100000)

        def side_leg(precision, seed, **extra):
            e = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=precision, **ekw, **extra)
            e.set_geometry(g)
            e.set_source(wl["source"])
            first = 0
            e.run(H64 // 4, nbatch=1, seed=seed, first=first)
            first += H64 // 4
            e.reset()
            torch.cuda.synchronize()
            start.record()
            for _ in range(2):
                flush.zero_()
                e.run(H64, nbatch=1, seed=seed, first=first)
                first += H64
            stop.record()
            torch.cuda.synchronize()
            t = start.elapsed_time(stop) / 1e3
            s_, s2_, _ = e.tallies()
            sig_, _ = sigma_eff(s_, s2_, 2)
            pr = e.profile()
            e.close()
            return t, (1.0 / (sig_ * sig_ * t) if sig_ else None), pr

        T64, eff64, _ = side_leg(64, seed0 + 2000)
        line["fp64"] = {"value": 2 * H64 / T64, "unit": "histories/s", "dose_efficiency": eff64,
                        "histories_per_step": H64, "steps": 2, "timing": "CUDA events"}
        if eff and eff64:
            line["efficiency_ratio_fp32_over_fp64"] = eff / eff64
        # the FP32 kernels with FP64 residual ranges and face distances near
        # voxel faces (egsgpu_config.fp64_near_faces), timed the same way
        Tnf, effnf, pnf = side_leg(32, seed0 + 2500, fp64_near_faces=1)
        line["fp64_near_faces"] = {
            "value": 2 * H64 / Tnf, "unit": "histories/s", "dose_efficiency": effnf, "histories_per_step": H64,
            "steps": 2, "timing": "CUDA events",
            "electron_steps_in_fp64": (pnf.get("electron_wide_steps", 0.0) / pnf["electron_steps"]
                                       if pnf.get("electron_steps") else 0.0),
            "efficiency_ratio_over_fp64": (effnf / eff64) if (effnf and eff64) else None}
        line["fp32_vs_fp64"] = fp32_vs_fp64(wl, eg, ekw, max(H // 100, 200000), seed0 + 3000)
    line["simt"] = simt_roofline(prof)
    line["clocks"] = clk.summary()
    if rank == 0 and ws == 1 and not args.no_batched and args.workload == "slab64":
        # the batched configuration (64 phantoms per launch sequence) beside the headline
        b = batched_measure(args, 1, 0, local, None, 3, 3, True, 0.05)
        keep = ("value", "unit", "ms_per_step", "config", "dose_efficiency", "sigma_bar_50pct", "e2e",
                "one_at_a_time", "fp64_one_at_a_time", "efficiency_ratio_batched_fp32_over_fp64", "gpu_launches",
                "autotuner")
        line["batched64"] = {k: b[k] for k in keep if k in b}
        line["batched64"]["steps"] = 3
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        n, dt = cpu_sample(wl, args.cpu_seconds, threads, seed0 + 4000)
        line["cpu_baseline"] = {"value": n / dt, "unit": "histories/s", "cores": threads, "kind": "port",
                                "sample": "%d histories of %s on %d host threads, %.1f s" % (n, wl["name"],
                                                                                          threads, dt)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
