#!/usr/bin/env python
"""Benchmark of the structured multiply on GB300: Cauchy A*C at n = 16384.

Workload (one step = one pass of the hot path over one batch): psmma_cauchy on the split
path, Q = A*H with H(i,j) = u_i v_j / (d_i - w_j), n = k = 16384, 10% of the poles within
1e-10 of a neighbour, A ~ N(0,1) in FP64; inputs resident in HBM (A is 2 GiB, larger
than L2, so no explicit flush is needed between steps).  Reported beside it:
  * the FP64 plain path (FP64 tensor-core MMA, H generated in shared memory) on the same
    inputs, and the relative Frobenius error of the split result against it and against
    the CPU oracle on sampled rows;
  * p50/p99 step latency, per-phase times (CUDA events on the launch stream);
  * e2e: the same metric through the host-pointer entry point psmma_cauchy_host with
    pinned host buffers, host<->device copies inside the timed region;
  * roofline of the dominant kernel (the modular BF16 GEMM, tensor-bound);
  * cpu_baseline: the oracle's restatement of the reference (ConstCauchy + DGEMM, which is
    what PSCAUCHY_COMPUTE does on a 1x1 process grid) on the host cores, on a row sample.

``python bench.py --impl reference`` times that CPU restatement alone (the reference is
Fortran + MPI + ScaLAPACK and cannot be built on this machine or the GPU host).
Multi-GPU (torchrun): each rank multiplies its own 16384-row panel of A by the same H
(weak scaling, no collective on the data path); value = total FLOPs / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Cauchy A·C eff. TFLOP/s n=16384, FP64 vs split-prec at ≤1e-12 err; p99 ms"
N_DEFAULT = 16384
CPU_COLS = 1024  # column-panel sample of the CPU baseline per step


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"bf16": d.get("bf16_tflops", 1900.0), "bf16_sustained": d.get("bf16_tflops_sustained", 1700.0),
                "hbm": d.get("hbm_gbs", 6800.0), "source": "measured"}
    return {"bf16": 1900.0, "bf16_sustained": 1700.0, "hbm": 6800.0, "source": "fallback"}


def ncu_traffic(n: int, nmod: int):
    """DRAM bytes per launch of the modular GEMM from the committed full-size ncu capture
    (profiles/crt_gemm_ncu.md), scaled by the moduli count (one plane pass per modulus)
    and, for other sizes, by n^3 (re-reads grow with the tile count times k)."""
    f = ROOT / "profiles" / "crt_gemm_ncu.md"
    if not f.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch_n(\d+)_m(\d+):\s*([0-9.eE+]+)", f.read_text())
    if not m:
        return None
    n0, m0, b0 = int(m.group(1)), int(m.group(2)), float(m.group(3))
    return b0 * (nmod / m0) * (n / n0) ** 3


def profile_traffic(tag: str):
    """DRAM bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum) recorded as
    ``traffic_bytes_per_launch_<tag>: <bytes>`` in a committed profile summary under
    profiles/, or None."""
    d = ROOT / "profiles"
    if not d.is_dir():
        return None
    pat = re.compile(r"traffic_bytes_per_launch_" + re.escape(tag) + r":\s*([0-9.eE+]+)")
    for f in sorted(d.glob("*.md")):
        m = pat.search(f.read_text())
        if m:
            return float(m.group(1))
    return None


class Clocks:
    """nvidia-smi clock/throttle sampling during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"psmma_bench_clocks_{os.getpid()}_{index}.csv"

    def start(self):
        try:
            self.path.parent.mkdir(exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        try:
            self.path.unlink()
        except Exception:
            pass
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl != "reference" else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, ws: int, device=None) -> float:
    if ws == 1:
        return x
    from psmma_git_gb300.shard import max_over_ranks as _max
    return _max(x)


def link_rates(h_buf, dev, nbytes: int = 512 << 20) -> dict:
    """Pinned host<->device copy rates (GB/s, best of 3) over the first nbytes of h_buf."""
    import torch
    h = h_buf.reshape(-1)[: nbytes // h_buf.element_size()]
    d = torch.empty_like(h, device=dev)
    out = {}
    for name, fn in (("h2d", lambda: d.copy_(h, non_blocking=True)),
                     ("d2h", lambda: h.copy_(d, non_blocking=True))):
        best = float("inf")
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        out[name] = round(h.numel() * h.element_size() / (best * 1e-3) / 1e9, 1)
    del d
    return out


def cpu_inputs(n: int, seed_gen: int = 0, seed_a: int = 1):
    import numpy as np
    from oracle import psmma_oracle as O
    gen = O.cfg_cauchy_generators(n, seed=seed_gen, clustered=0.1)
    rng = np.random.Generator(np.random.PCG64(seed_a))
    A = np.asfortranarray(rng.standard_normal((n, n)))
    return A, gen


def cpu_sample(A, gen, cols: int):
    """One bounded step of the CPU restatement: the column panel Q[:, 0:cols] = A * H[:, 0:cols]
    -- ConstCauchy of that panel of H followed by one DGEMM, i.e. what PSCAUCHY_COMPUTE does
    for the first ring step of one process column (every part of the work scales by
    cols / n)."""
    import numpy as np
    from oracle import psmma_oracle as O
    n, k = A.shape
    t0 = time.perf_counter()
    H = O.const_cauchy(gen, np.arange(1, k + 1), np.arange(1, cols + 1))
    Qp = A @ H
    return time.perf_counter() - t0, Qp


def run_reference(args, ws, rank):
    if rank != 0:
        return 0
    n = args.n
    cols = args.cpu_cols
    A, gen = cpu_inputs(n)
    for _ in range(args.warmup):
        cpu_sample(A, gen, cols)
    times = []
    for _ in range(args.steps):
        t, _ = cpu_sample(A, gen, cols)
        times.append(t)
    tot = sum(times)
    flops = 2.0 * n * n * cols * args.steps
    val = flops / tot / 1e12
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "TFLOP/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"psmma_cauchy n={n} clustered poles, CPU restatement of PSCAUCHY_COMPUTE "
                               f"(ConstCauchy + DGEMM), column panel {n} x {cols} of Q per step", "n": n, "k": n},
        "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"Q[:, 0:{cols}] of the {n}x{n} product per step (H panel generated each step)"},
        "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "latency_ms": {"p50": 1e3 * statistics.median(times), "p99": 1e3 * max(times)},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, ws, rank, local):
    import numpy as np
    import torch
    import psmma_git_gb300 as P
    from psmma_git_gb300 import _lib
    from oracle import psmma_oracle as O

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.load()
    n = k = args.n
    stream = torch.cuda.current_stream(dev)

    gen_np = O.cfg_cauchy_generators(k, seed=0, clustered=0.1)
    gen = torch.from_numpy(np.ascontiguousarray(gen_np.T)).to(dev).t()
    g = torch.Generator(device=dev)
    g.manual_seed(1 + rank)
    if args.strong:
        # one n x k problem split in row panels over the ranks (shard.sharded_multiply): each
        # rank holds and multiplies rows [lo, hi) only; the headline's side measurements
        # (FP64 path, e2e, CPU baseline, other workloads) are skipped
        from psmma_git_gb300.shard import local_panel, sharded_multiply
        lo, hi = local_panel(n, rank, ws)
        args.no_fp64 = args.no_e2e = args.no_cpu = args.no_extra = True
        g.manual_seed(1)
        A_full_rows = torch.randn(k, hi - lo, generator=g, device=dev, dtype=torch.float64)
        n_rank = hi - lo
    else:
        n_rank = n
    A = P.fortran_empty(n_rank, k, torch.float64, dev)
    A.copy_(A_full_rows.t() if args.strong else torch.randn(k, n, generator=g, device=dev, dtype=torch.float64).t())
    Q = P.fortran_empty(n_rank, k, torch.float64, dev)
    Q.zero_()

    def step():
        if args.strong:
            sharded_multiply("cauchy", n, k, 1.0, A, gen, 0.0, Q, rank=rank, world=ws, precision="split",
                             n_moduli=args.n_moduli, stream=stream)
        else:
            P.psmma_cauchy(n, k, 1.0, A, gen, 0.0, Q, precision="split", n_moduli=args.n_moduli, stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # ---------------- timed region (split path): calls back to back, no tracing ----------------
    clocks = Clocks(local)
    clocks.start()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    barrier(ws)
    torch.cuda.synchronize()
    ev[0].record(stream)
    for s in range(args.steps):
        step()
        ev[s + 1].record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    cl = clocks.stop()
    # ---------------- per-phase trace: the same number of steps again, one event per phase ----
    lib.psmma_set_profiling(1)
    phase_tot = {}
    for s in range(args.steps):
        step()
        ms = (C_float * 16)()
        names = (C_charp * 16)()
        m = lib.psmma_profile_read(ms, names, 16)
        for i in range(m):
            phase_tot[names[i].decode()] = phase_tot.get(names[i].decode(), 0.0) + ms[i]
    lib.psmma_set_profiling(0)
    step_ms = [ev[s].elapsed_time(ev[s + 1]) for s in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[args.steps])
    total_ms = max_over_ranks(total_ms, ws, dev)
    flops_rank = 2.0 * n * k * k
    flops_job = flops_rank if args.strong else flops_rank * ws  # strong: one problem over all ranks
    value = flops_job * args.steps / (total_ms * 1e-3) / 1e12
    phases = {kname: v / args.steps for kname, v in phase_tot.items()}
    launches_per_step = len(phases) + 1  # one kernel per phase + the stream-status accumulation

    result = {"metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
              "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
              "scaling": "strong" if args.strong else "weak", "vs_baseline": None, "dtype": "bf16",
              "data": "synthetic"}
    result["config"] = {
        "workload": f"psmma_cauchy split-precision n={n} (10% of poles within 1e-10 of a neighbour, A ~ N(0,1) FP64)",
        "n": n, "k": k, "kind": "cauchy", "precision": "split (CRT residues on BF16 tcgen05, FP64 recombination)",
        "n_moduli": args.n_moduli, "l2": "inputs larger than L2 (A = 2 GiB), no flush",
        "parallelism": (f"one problem in {ws} row panel(s) of {n_rank}+ rows, no collective" if args.strong
                        else f"{ws} replica(s), row panels, no collective")}
    result["latency_ms"] = {"p50": statistics.median(step_ms),
                            "p99": float(np.percentile(np.asarray(step_ms), 99))}
    result["phases_ms"] = phases
    result["gpu_launches"] = launches_per_step * args.steps

    # ---------------- roofline of the modular GEMM ----------------
    pk = peaks()
    gemm_ms = phases.get("modular_gemm")
    kp = (k + 63) // 64 * 64
    if gemm_ms:
        flops_gemm = 2.0 * args.n_moduli * n * k * kp
        achieved = flops_gemm / (gemm_ms * 1e-3) / 1e12
        traffic = ncu_traffic(n, args.n_moduli)
        result["roofline"] = {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_sustained"],
                              "unit": "TFLOP/s", "frac": achieved / pk["bf16_sustained"], "traffic": traffic,
                              "kernel": "k_crt_gemm", "flops_per_launch": flops_gemm,
                              "peak_note": f"{pk['source']} cuBLAS bf16 sustained (kernel timed inside a "
                                           f"multi-second loop); burst {pk['bf16']}",
                              "frac_of_burst": achieved / pk["bf16"],
                              "traffic_note": "DRAM bytes per launch from the one-pass ncu capture at n=16384, "
                                              "13 moduli (profiles/crt_gemm_ncu.md), scaled by moduli and n^3; "
                                              "not measured in this run"}

    if rank == 0:
        # ---------------- FP64 plain path on the same inputs ----------------
        if not args.no_fp64:
            Q64 = P.fortran_empty(n, k, torch.float64, dev)
            A_small = A[:2048, :2048]
            P.psmma_cauchy(2048, 2048, 1.0, A_small, gen[:2048], 0.0, Q64[:2048, :2048], stream=stream)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            P.psmma_cauchy(n, k, 1.0, A, gen, 0.0, Q64, precision="fp64", stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            t64 = e0.elapsed_time(e1)
            # cuBLAS DGEMM rate on this GPU, the FP64 roofline denominator
            a = torch.randn(8192, 8192, device=dev, dtype=torch.float64)
            torch.matmul(a, a)
            torch.cuda.synchronize()
            e0.record(stream)
            torch.matmul(a, a)
            e1.record(stream)
            torch.cuda.synchronize()
            dgemm = 2 * 8192 ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12
            del a
            v64 = flops_rank / (t64 * 1e-3) / 1e12
            rel = (torch.linalg.norm(Q - Q64) / torch.linalg.norm(Q64)).item()
            result["fp64_plain"] = {"value": v64, "unit": "TFLOP/s", "ms_per_step": t64, "steps": 1,
                                    "cublas_dgemm_tflops": dgemm, "frac_of_dgemm": v64 / dgemm,
                                    "speedup_split_vs_fp64": value / ws / v64}
            result["rel_err"] = {"split_vs_fp64_path": rel}
            del Q64
        # ---------------- e2e through the host-pointer entry point ----------------
        # (before the CPU baseline, whose BLAS threads would otherwise still compete for the
        # host cores that issue the copies and launches)
        e2e_done = False
        if not args.no_e2e:
            hA = torch.empty((k, n), dtype=torch.float64, pin_memory=True)
            hA.copy_(A.t())
            hQ = torch.empty((k, n), dtype=torch.float64, pin_memory=True)
            hG = torch.empty((4, k), dtype=torch.float64, pin_memory=True)
            hG.copy_(gen.t())
            nA, nQ, nG = hA.numpy().T, hQ.numpy().T, hG.numpy().T
            del A, Q
            torch.cuda.empty_cache()
            # warm-up calls: the first of a shape picks the bit counts the later ones speculate
            # with; the first speculative call also pays a one-time cost of the pitched row-panel
            # uploads (about 20 ms on the first panel)
            for _ in range(max(2, args.warmup)):
                P.psmma_cauchy(n, k, 1.0, nA, nG, 0.0, nQ, precision="split", n_moduli=args.n_moduli)
            e2e_steps = max(1, min(args.steps, 10))
            call_ms, dev_ms, redo, first_phases, slow, timelines = [], [], 0, None, (0.0, None, None), []
            # each call is traced (one event per library phase, no synchronisation added): the
            # device-side span of the call and whether its speculative bit counts were redone
            lib.psmma_set_profiling(1)
            t0 = time.perf_counter()
            for _ in range(e2e_steps):
                t1 = time.perf_counter()
                P.psmma_cauchy(n, k, 1.0, nA, nG, 0.0, nQ, precision="split", n_moduli=args.n_moduli)
                call_ms.append(round((time.perf_counter() - t1) * 1e3, 2))
                ms = (C_float * 80)()
                names = (C_charp * 80)()
                m = lib.psmma_profile_read(ms, names, 80)
                dev_ms.append(round(sum(ms[j] for j in range(max(0, m))), 2))
                ph = [[names[j].decode(), round(ms[j], 3)] for j in range(max(0, m))]
                mt = lib.psmma_profile_read_timeline(ms, names, 80)
                tl = [[names[j].decode(), round(ms[j], 2)] for j in range(max(0, mt))]
                if first_phases is None:
                    first_phases = ph
                if dev_ms[-1] > slow[0]:
                    slow = (dev_ms[-1], ph, tl)
                timelines.append(tl)
                redo += any(names[j] == b"redo_wrong_guess" for j in range(max(0, m)))
            te = (time.perf_counter() - t0) / e2e_steps
            lib.psmma_set_profiling(0)
            result["e2e"] = {"value": flops_rank / te / 1e12, "unit": "TFLOP/s",
                             "h2d_bytes_per_step": n * k * 8 + 4 * k * 8, "d2h_bytes_per_step": n * k * 8,
                             "ms_per_step": te * 1e3, "steps": e2e_steps, "call_ms": call_ms,
                             # the mean above keeps every call; these show how much of it is
                             # the host link's stalls (calls above 1.25x the median)
                             "median_call_tflops": flops_rank / (statistics.median(call_ms) * 1e-3) / 1e12,
                             "stalled_calls": sum(c > 1.25 * statistics.median(call_ms) for c in call_ms),
                             "device_span_ms": dev_ms, "redone_calls": redo, "first_call_phases_ms": first_phases,
                             "slowest_call_phases_ms": slow[1],
                             "slowest_call_timeline_ms": slow[2],
                             "upload_done_ms": [[v for nm, v in tl if nm == "a_panel_up"] for tl in timelines],
                             "api": "psmma_cauchy_host (pinned host buffers)"}
            # after the timed calls: one traced call (library-stream phases) and the pinned
            # copy rate of this host link, which bound the end-to-end time from below
            lib.psmma_set_profiling(1)
            P.psmma_cauchy(n, k, 1.0, nA, nG, 0.0, nQ, precision="split", n_moduli=args.n_moduli)
            ms = (C_float * 40)()
            names = (C_charp * 40)()
            m = lib.psmma_profile_read(ms, names, 40)
            lib.psmma_set_profiling(0)
            result["e2e"]["phases_ms"] = [[names[j].decode(), round(ms[j], 3)] for j in range(max(0, m))]
            result["e2e"]["link_gbs"] = link_rates(hA, dev)
            e2e_done = True
        # ---------------- CPU baseline + oracle panel ----------------
        if not args.no_cpu:
            # (after the e2e leg the operands live in its pinned host buffers, and Q holds the
            # same product computed through the host-pointer entry point)
            Acpu = np.asfortranarray(nA) if e2e_done else np.asfortranarray(A.t().contiguous().cpu().numpy().T)
            t, Qcpu = cpu_sample(Acpu, gen_np, args.cpu_cols)
            del Acpu
            cpu_val = 2.0 * n * k * args.cpu_cols / t / 1e12
            result["cpu_baseline"] = {"value": cpu_val, "unit": "TFLOP/s", "cores": os.cpu_count(),
                                      "kind": "port",
                                      "sample": f"Q[:, 0:{args.cpu_cols}] of the {n}x{n} product: ConstCauchy of "
                                                f"that H panel + DGEMM (oracle restatement), {t:.1f} s"}
            got = (np.asarray(nQ[:, :args.cpu_cols]) if e2e_done
                   else Q[:, :args.cpu_cols].t().contiguous().cpu().numpy().T)
            result.setdefault("rel_err", {})["split_vs_cpu_oracle_panel"] = O.rel_fro(got, Qcpu)
        if cl is not None:
            result["clocks"] = cl
        if not args.no_extra:
            result["extra"] = run_extras(args, ws, rank, local)
        print(json.dumps(result), flush=True)
    return 0


def run_case(args, ws, rank, local):
    """One workload repeated, for profiling a kernel on a small case (``--case PREC:KIND``,
    PREC fp64 or split, KIND cauchy / toeplitz / hankel / dft / cauchyeig, size --n): warm-up
    calls, then --steps calls timed with CUDA events.  Inputs as the cfg0 / cfg1 workloads.
    One JSON line with the mean time per call."""
    import numpy as np
    import torch
    import psmma_git_gb300 as P
    from oracle import psmma_oracle as O
    if rank != 0:
        return 0
    prec, kind = args.case.split(":")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = k = args.n
    g = torch.Generator(device=dev)
    g.manual_seed(9)
    col = lambda x: torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(dev).t()  # noqa: E731
    if kind == "dft":
        X = P.fortran_empty(n, k, torch.complex128, dev)
        X.copy_(torch.complex(torch.rand(k, n, generator=g, device=dev, dtype=torch.float64) * 2 - 1,
                              torch.rand(k, n, generator=g, device=dev, dtype=torch.float64) * 2 - 1).t())
        Y = P.fortran_empty(n, k, torch.complex128, dev)
        run = lambda: P.pzmdftl(n, k, 1.0, X, 0.0, Y, precision=prec, n_moduli=args.n_moduli)  # noqa: E731
        flops = 8.0 * n ** 3
    else:
        A = P.fortran_empty(n, k, torch.float64, dev)
        A.copy_(torch.rand(k, n, generator=g, device=dev, dtype=torch.float64).mul_(2).sub_(1).t())
        Y = P.fortran_empty(n, k, torch.float64, dev)
        flops = 2.0 * n ** 3
        if kind == "cauchy":
            gen = col(O.cfg_cauchy_generators(k, seed=0))
            run = lambda: P.psmma_cauchy(n, k, 1.0, A, gen, 0.0, Y, precision=prec, n_moduli=args.n_moduli)  # noqa: E731
        elif kind == "cauchyeig":
            eig = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in O.eig_generators(k, seed=7, tiny=k // 100)]
            run = lambda: P.psmma_cauchyeig(n, k, 1.0, A, *eig, 0.0, Y, precision=prec,  # noqa: E731
                                            n_moduli=args.n_moduli)
        else:
            gv = torch.rand(2 * k - 1, generator=g, device=dev, dtype=torch.float64).mul_(2).sub_(1)
            fn = P.psmma_toeplitz if kind == "toeplitz" else P.psmma_hankel
            run = lambda: fn(n, k, 1.0, A, gv, 0.0, Y, precision=prec, n_moduli=args.n_moduli)  # noqa: E731
    for _ in range(args.warmup):
        run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        run()
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / args.steps
    # the timed result checked on a sample: 4 columns against the FFT (DFT), or 64 rows against
    # the FP64 path (the other kinds)
    if kind == "dft":
        ref = np.fft.fft(X[:, :4].cpu().numpy(), axis=0)
        err = O.rel_fro(Y[:, :4].cpu().numpy(), ref)
    else:
        R64 = P.fortran_empty(64, k, torch.float64, dev)
        if kind == "cauchy":
            P.psmma_cauchy(64, k, 1.0, A[:64], gen, 0.0, R64)
        elif kind == "cauchyeig":
            P.psmma_cauchyeig(64, k, 1.0, A[:64], *eig, 0.0, R64)
        else:
            fn(64, k, 1.0, A[:64], gv, 0.0, R64)
        torch.cuda.synchronize()
        err = float(torch.linalg.norm(Y[:64] - R64) / torch.linalg.norm(R64))
    print(json.dumps({"case": args.case, "n": n, "ms_per_call": t, "tflops": flops / t / 1e9,
                      "steps": args.steps, "warmup": args.warmup, "rel_err_sample": err}), flush=True)
    return 0 if err < (1e-12 if prec == "split" else 1e-13) else 1


def run_extras(args, ws, rank, local) -> dict:
    """The other workloads of the benchmark, each in compact form, for the same JSON line (after
    the headline's timed region, which they do not touch):
      cfg0  FP64 Cauchy n = 2048, seeds 0..4 (roofline vs in-run DGEMM, e2e, CPU ring baseline);
      cfg1  Toeplitz / Hankel / DFT / CAUCHYEIG n = 8192 on both paths (rooflines, CPU panels);
      cfg3  the batched merge level, 64 problems (RRQR, RRLU, Toeplitz RRQR; GEMM and QR rooflines);
      cfg4  a serving sweep (p50 / p99 per rate against the stated bound, saturation).
    Each runs with its own fixed step counts (a few minutes in all); a failure is recorded in
    its entry and does not stop the others."""
    import copy
    import torch
    import psmma_git_gb300 as P
    out = {}
    plan = [
        ("cfg0", run_cfg0, dict(steps=10, warmup=3)),
        ("cfg1", run_cfg1, dict(steps=5, warmup=3)),
        ("cfg3", run_merge_level, dict(steps=5, warmup=3, no_tune=False)),
        ("cfg4", run_serving, dict(rates=[20.0, 40.0, 60.0], serve_seconds=4.0)),
    ]
    for name, fn, over in plan:
        a = copy.copy(args)
        for kk, vv in over.items():
            setattr(a, kk, vv)
        t0 = time.perf_counter()
        try:
            line = fn(a, ws, rank, local, compact=True)
            if line is not None:
                line = {kk: vv for kk, vv in line.items() if kk not in ("n_gpus", "data")}
        except Exception as e:  # noqa: BLE001 - recorded in the line, the headline still prints
            line = {"error": f"{type(e).__name__}: {e}"}
        line["wall_s"] = round(time.perf_counter() - t0, 1)
        out[name] = line
        print(json.dumps({"extra_done": name, "wall_s": line["wall_s"]}), file=sys.stderr, flush=True)
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        P.load().psmma_release_workspace()  # the library's per-stream pools of this workload
    return out


def run_serving(args, ws, rank, local, compact=False):
    """Serving loop under a Poisson request stream (one line of JSON per sweep).  Requests:
    kind uniform over cauchy/toeplitz/hankel/dft, n log-uniform in [512, 16384] (k = n),
    operands uniform[-1,1] resident on the device (views into pre-generated pools), split
    precision; the server admits by an HBM budget with at most --inflight requests.  Reported
    per rate: p50/p99 latency, throughput, whether p99 holds the stated bound; over the sweep:
    the largest rate that holds it and the saturation throughput (the largest measured).
    Returns the JSON object."""
    import math
    import threading
    import numpy as np
    import torch
    import psmma_git_gb300 as P
    from psmma_git_gb300.server import Server
    from oracle import psmma_oracle as O
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    nmax = args.serve_nmax
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    A = P.fortran_empty(nmax, nmax, torch.float64, dev)
    A.copy_(torch.rand(nmax, nmax, generator=g, device=dev, dtype=torch.float64).mul_(2).sub_(1))
    B = P.fortran_empty(nmax, nmax, torch.complex128, dev)
    B.copy_(torch.complex(torch.rand(nmax, nmax, generator=g, device=dev, dtype=torch.float64) * 2 - 1,
                          torch.rand(nmax, nmax, generator=g, device=dev, dtype=torch.float64) * 2 - 1))
    gen_c = torch.from_numpy(np.ascontiguousarray(O.cfg_cauchy_generators(nmax, seed=0).T)).to(dev).t()
    gvec = torch.rand(2 * nmax - 1, generator=g, device=dev, dtype=torch.float64).mul_(2).sub_(1)
    nbuf = args.inflight * 3
    # flat pools: viewed per request as a column-major n x n real or complex matrix
    outs = [torch.empty(2 * nmax * nmax, dtype=torch.float64, device=dev) for _ in range(nbuf)]
    kinds = ["cauchy", "toeplitz", "hankel", "dft"]
    budget = args.serve_budget_gib << 30
    results = []
    for rate in args.rates:
        rng = np.random.default_rng(int(rate * 1000) + 1)
        n_req = max(8, int(rate * args.serve_seconds))
        plan = []
        t = 0.0
        for i in range(n_req):
            t += rng.exponential(1.0 / rate)
            n = int(round(math.exp(rng.uniform(math.log(512), math.log(nmax)))))
            plan.append((t, kinds[int(rng.integers(4))], n))
        buf_ticket = [None] * nbuf
        tickets, lat, flops, done = [], [], [], []
        with Server(budget, max_inflight=args.inflight) as srv:
            lock = threading.Lock()

            def collect(tk, fl):
                info = srv.wait(tk)
                with lock:
                    done.append((info, fl))

            threads = []
            t0 = time.perf_counter()
            for i, (ta, kind, n) in enumerate(plan):
                b = i % nbuf
                if buf_ticket[b] is not None:
                    buf_ticket[b].join()  # its previous request must be complete
                while time.perf_counter() - t0 < ta:
                    time.sleep(min(0.001, max(0.0, ta - (time.perf_counter() - t0))))
                if kind == "dft":
                    Q = torch.view_as_complex(outs[b][: 2 * n * n].view(n, n, 2)).t()
                    tk = srv.submit("dft", n, n, 1.0, B[:n, :n], None, 0.0, Q, precision="split",
                                    n_moduli=args.n_moduli, tag=i)
                    fl = 8.0 * n ** 3
                else:
                    Q = outs[b][: n * n].view(n, n).t()
                    gen = gen_c[:n] if kind == "cauchy" else gvec[: 2 * n - 1]
                    tk = srv.submit(kind, n, n, 1.0, A[:n, :n], gen, 0.0, Q, precision="split",
                                    n_moduli=args.n_moduli, tag=i)
                    fl = 2.0 * n ** 3
                th = threading.Thread(target=collect, args=(tk, fl))
                th.start()
                buf_ticket[b] = th
                threads.append(th)
            for th in threads:
                th.join()
            wall = max(i["end_s"] for i, _ in done) - min(i["submit_s"] for i, _ in done)
        ok = all(i["status"] == 0 for i, _ in done)
        lats = np.array([i["latency_s"] for i, _ in done]) * 1e3
        tot_fl = sum(f for _, f in done)
        results.append({"rate_req_s": rate, "requests": len(done), "all_ok": ok,
                        "throughput_req_s": len(done) / wall, "throughput_tflops": tot_fl / wall / 1e12,
                        "p50_ms": float(np.percentile(lats, 50)), "p99_ms": float(np.percentile(lats, 99)),
                        "max_ms": float(lats.max()),
                        "mean_gpu_ms": float(np.mean([i["gpu_ms"] for i, _ in done])),
                        "p99_within_bound": bool(np.percentile(lats, 99) < args.p99_bound_ms)})
        print(json.dumps({"serving_rate": results[-1]}), file=sys.stderr, flush=True)
    # the largest rate up to which every measured rate held the bound
    held = []
    for r in sorted(results, key=lambda r: r["rate_req_s"]):
        if not (r["p99_within_bound"] and r["all_ok"]):
            break
        held.append(r["rate_req_s"])
    line = {"metric": "serving: p50/p99 latency (ms) and effective TFLOP/s under a Poisson stream",
            "unit": "ms", "n_gpus": 1, "data": "synthetic",
            "config": {"workload": "kind uniform over cauchy/toeplitz/hankel/dft, n log-uniform in "
                                   f"[512, {nmax}], split precision ({args.n_moduli} moduli), device-resident "
                                   "operands", "hbm_budget_gib": args.serve_budget_gib,
                       "max_inflight": args.inflight, "seconds_per_rate": args.serve_seconds},
            "p99_bound_ms": args.p99_bound_ms, "sweep": results,
            "largest_rate_within_bound_req_s": held[-1] if held else None,
            "rates_within_bound_req_s": [r["rate_req_s"] for r in results if r["p99_within_bound"] and r["all_ok"]],
            "saturation_tflops": max(r["throughput_tflops"] for r in results),
            "all_ok": all(r["all_ok"] for r in results)}
    return line


def run_cfg1(args, ws, rank, local, compact=False):
    """Toeplitz, Hankel, DFT and accurate-denominator Cauchy (PSMMA_CAUCHYEIG) multiplies at
    n = k = 8192 (A uniform[-1,1], generator vector of length 2n-1 uniform[-1,1]; DFT: complex
    B with both parts uniform[-1,1]; CAUCHYEIG: eigensolver generators with 1% of the roots next
    to their pole) on the split path (args.n_moduli) and the FP64 path.  Rates: 2n^3/t for
    Toeplitz/Hankel/CAUCHYEIG, 8n^3/t real flops for the DFT (2n^3/t complex multiply-adds
    beside it).  Errors: split vs FP64 path on the whole product, and both against the
    oracle on a 256-row (DFT: 256-column) sample -- FFT correlation for Toeplitz/Hankel, FFT for
    the DFT, the explicit CauchylikeEig matrix (FP64 BLAS) for CAUCHYEIG, whose per-column
    maximum relative error is reported too (the eigensolver normalises columns).  Per kind a
    roofline of the modular GEMMs (BF16, sustained peak) and of the FP64 path (in-run DGEMM),
    and a CPU baseline: the oracle's restatement (ConstToeplitz / ConstHankel / CauchylikeEig
    of an H column panel + DGEMM; the DFT: a row panel of F times B by ZGEMM) on all host
    cores.  Returns the JSON object."""
    import numpy as np
    import torch
    import psmma_git_gb300 as P
    from oracle import psmma_oracle as O
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = k = args.cfg1_n
    nmod = args.n_moduli
    pk = peaks()
    stream = torch.cuda.current_stream()
    dgemm = fp64_dgemm_rate(dev, stream)
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    A = P.fortran_empty(n, k, torch.float64, dev)
    A.copy_(torch.rand(k, n, generator=g, device=dev, dtype=torch.float64).mul_(2).sub_(1).t())
    gv = torch.rand(2 * k - 1, generator=g, device=dev, dtype=torch.float64).mul_(2).sub_(1)
    out = {}
    eig = O.eig_generators(k, seed=7, tiny=k // 100)  # F, U, V, DIFL, DIFR (1% of roots next to a pole)
    eig_dev = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for x in eig]
    A_host = None
    cpu_cols = 512 if not compact else 256
    kp = (k + 63) // 64 * 64
    for kind in ["toeplitz", "hankel", "dft", "cauchyeig"]:
        if kind == "cauchyeig":
            Y = P.fortran_empty(n, k, torch.float64, dev)
            Y64 = P.fortran_empty(n, k, torch.float64, dev)
            run = lambda prec, dst: P.psmma_cauchyeig(n, k, 1.0, A, *eig_dev, 0.0, dst, precision=prec,  # noqa: E731
                                                      n_moduli=nmod)
            flops = 2.0 * n ** 3
            gemm_flops = 2.0 * nmod * n * k * kp
        elif kind == "dft":
            X = P.fortran_empty(n, k, torch.complex128, dev)
            X.copy_(torch.complex(torch.rand(k, n, generator=g, device=dev, dtype=torch.float64) * 2 - 1,
                                  torch.rand(k, n, generator=g, device=dev, dtype=torch.float64) * 2 - 1).t())
            Y = P.fortran_empty(n, k, torch.complex128, dev)
            Y64 = P.fortran_empty(n, k, torch.complex128, dev)
            run = lambda prec, dst: P.pzmdftl(n, k, 1.0, X, 0.0, dst, precision=prec, n_moduli=nmod)  # noqa: E731
            flops = 8.0 * n ** 3
            # 3M: three real products per modulus, on F_(n/R) and R k columns (radix-R first step)
            R = P.load().psmma_split_dft_radix(n)
            kq = (n // R + 63) // 64 * 64
            gemm_flops = 3 * 2.0 * nmod * (R * k) * (n // R) * kq
        else:
            Y = P.fortran_empty(n, k, torch.float64, dev)
            Y64 = P.fortran_empty(n, k, torch.float64, dev)
            fn = P.psmma_toeplitz if kind == "toeplitz" else P.psmma_hankel
            run = lambda prec, dst, fn=fn: fn(n, k, 1.0, A, gv, 0.0, dst, precision=prec, n_moduli=nmod)  # noqa: E731
            flops = 2.0 * n ** 3
            # the block step (automatic levels L): 3^L modular products of width w = k / 2^L
            levels = P.load().psmma_split_block_levels(1 if kind == "toeplitz" else 2, n, k)
            w = k >> levels
            gemm_flops = 2.0 * nmod * n * w * ((w + 63) // 64 * 64) * 3 ** levels
        for _ in range(args.warmup):
            run("split", Y)
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
        e[0].record()
        for i in range(args.steps):
            run("split", Y)
            e[i + 1].record()
        torch.cuda.synchronize()
        t = e[0].elapsed_time(e[args.steps]) / args.steps
        # one traced call after the timed ones: the split path's phases
        lib = P.load()
        lib.psmma_set_profiling(1)
        run("split", Y)
        ms = (ctypes.c_float * 40)()
        names = (ctypes.c_char_p * 40)()
        m = lib.psmma_profile_read(ms, names, 40)
        lib.psmma_set_profiling(0)
        phases = [[names[j].decode(), round(ms[j], 3)] for j in range(max(0, m))]
        gemm_ms = sum(v for nm, v in phases if "gemm" in nm)
        e2e = None
        if kind in ("toeplitz", "hankel"):
            # end to end through the host-pointer entry point (pinned host A, generator and Q;
            # the copies inside each call, overlapped with the block step's row panels)
            hA = torch.empty((k, n), dtype=torch.float64, pin_memory=True)
            hA.copy_(A.t())
            hQ = torch.empty((k, n), dtype=torch.float64, pin_memory=True)
            hg = torch.empty(2 * k - 1, dtype=torch.float64, pin_memory=True)
            hg.copy_(gv)
            nA, nQ, ng = hA.numpy().T, hQ.numpy().T, hg.numpy()
            hfn = P.psmma_toeplitz if kind == "toeplitz" else P.psmma_hankel
            for _ in range(3):  # the first call of the shape picks the bit counts the others speculate with
                hfn(n, k, 1.0, nA, ng, 0.0, nQ, precision="split", n_moduli=nmod)
            t0 = time.perf_counter()
            for _ in range(args.steps):
                hfn(n, k, 1.0, nA, ng, 0.0, nQ, precision="split", n_moduli=nmod)
            te = (time.perf_counter() - t0) / args.steps
            e2e = {"value": flops / te / 1e12, "unit": "TFLOP/s", "ms_per_step": te * 1e3,
                   "h2d_bytes_per_step": n * k * 8 + (2 * k - 1) * 8, "d2h_bytes_per_step": n * k * 8,
                   "api": f"psmma_{kind}_host (pinned host buffers)",
                   "same_as_device_result": bool(torch.equal(torch.from_numpy(nQ.T.copy()).t().to(dev), Y))}
            del hA, hQ, hg
        run("fp64", Y64)  # warm-up (FP64 path: one call)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        run("fp64", Y64)
        e1.record()
        torch.cuda.synchronize()
        t64 = e0.elapsed_time(e1)
        rel = float(torch.linalg.norm(Y - Y64) / torch.linalg.norm(Y64))
        R64 = P.load().psmma_split_dft_radix(n) if kind == "dft" else 1  # the FP64 path takes the same step
        col_err = None
        if kind == "cauchyeig":
            As = np.ascontiguousarray(A[:256].cpu().numpy())
            ref = As @ O.cauchy_like_eig(*eig)
            err_split = O.rel_fro(Y[:256].cpu().numpy(), ref)
            err_64 = O.rel_fro(Y64[:256].cpu().numpy(), ref)
            col_err = {"split": O.col_max_rel(Y[:256].cpu().numpy(), ref),
                       "fp64": O.col_max_rel(Y64[:256].cpu().numpy(), ref)}
            oracle = "A[0:256] @ CauchylikeEig matrix (FP64 BLAS)"
        elif kind == "dft":
            Xs = X[:, :256].cpu().numpy()
            ref = O.dft_product(1.0, Xs, 0.0, None)
            err_split = O.rel_fro(Y[:, :256].cpu().numpy(), ref)
            err_64 = O.rel_fro(Y64[:, :256].cpu().numpy(), ref)
            oracle = "np.fft.fft of B[:, 0:256]"
        else:
            As = np.ascontiguousarray(A[:256].cpu().numpy())
            prod = O.toeplitz_product_fft if kind == "toeplitz" else O.hankel_product_fft
            ref = prod(As, gv.cpu().numpy(), k)
            err_split = O.rel_fro(Y[:256].cpu().numpy(), ref)
            err_64 = O.rel_fro(Y64[:256].cpu().numpy(), ref)
            oracle = "FFT correlation of A[0:256] with G"
        # CPU baseline: a bounded panel of the oracle's restatement on the host cores
        if A_host is None and not args.no_cpu:
            A_host = np.asfortranarray(A.cpu().numpy())
        cpu = None
        if not args.no_cpu:
            if kind == "dft":
                rows = 128 if compact else 256
                Bh = np.asfortranarray(X.cpu().numpy())
                t0 = time.perf_counter()
                jj = np.arange(rows, dtype=np.int64)[:, None] * np.arange(n, dtype=np.int64)[None, :] % n
                Fp = np.exp(-2j * np.pi * jj / n)
                Cp = Fp @ Bh
                tc = time.perf_counter() - t0
                del Bh, Fp, Cp
                cpu = {"value": 8.0 * rows * n * k / tc / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(),
                       "kind": "port", "sample": f"C[0:{rows}, :] = F[0:{rows}, :] @ B (F row panel generated "
                                                 f"+ ZGEMM), {tc:.2f} s"}
            else:
                cols = np.arange(1, cpu_cols + 1)
                t0 = time.perf_counter()
                if kind == "cauchyeig":
                    Hp = O.cauchy_like_eig(*eig, cindex=cols)
                else:
                    const = O.const_toeplitz if kind == "toeplitz" else O.const_hankel
                    Hp = const(gv.cpu().numpy(), k, np.arange(1, k + 1), cols)
                Qp = A_host @ Hp
                tc = time.perf_counter() - t0
                del Hp, Qp
                cpu = {"value": 2.0 * n * k * cpu_cols / tc / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(),
                       "kind": "port", "sample": f"Q[:, 0:{cpu_cols}]: the H column panel by the oracle's "
                                                 f"restatement + DGEMM, {tc:.2f} s"}
        out[kind] = {"split_ms": t, "split_tflops": flops / t / 1e9, "fp64_ms": t64,
                     "fp64_tflops": flops / t64 / 1e9, "speedup": t64 / t,
                     "rel_err_split_vs_fp64": rel, "rel_err_split_vs_oracle_sample": err_split,
                     "rel_err_fp64_vs_oracle_sample": err_64, "oracle": oracle,
                     "roofline": {"bound": "tensor", "achieved": gemm_flops / (gemm_ms * 1e-3) / 1e12 if gemm_ms
                                  else None, "peak": pk["bf16_sustained"], "unit": "TFLOP/s",
                                  "frac": gemm_flops / (gemm_ms * 1e-3) / 1e12 / pk["bf16_sustained"]
                                  if gemm_ms else None, "traffic": None, "kernel": "k_crt_gemm (modular BF16 GEMMs)",
                                  "flops_per_call": gemm_flops,
                                  "peak_note": f"{pk['source']} cuBLAS bf16 sustained"},
                     "fp64_roofline": {"bound": "tensor", "achieved": flops / R64 / t64 / 1e9, "peak": dgemm,
                                       "unit": "TFLOP/s", "frac": flops / R64 / t64 / 1e9 / dgemm,
                                       "kernel": "k_struct_f64",
                                       "peak_source": "cuBLAS DGEMM in this run; executed flops (the DFT's "
                                                      "radix step runs 1/R of the dense flops)"},
                     "cpu_baseline": cpu, "split_phases_ms": phases}
        if col_err is not None:
            out[kind]["col_max_rel_err_vs_oracle_sample"] = col_err
        if e2e is not None:
            out[kind]["e2e"] = e2e
        if kind in ("toeplitz", "hankel"):
            out[kind]["block_levels"] = levels
            out[kind]["executed_tflops"] = flops * 0.75 ** levels / t / 1e9
        if kind == "dft":
            out[kind]["split_complex_mac_tflops"] = 2.0 * n ** 3 / t / 1e9
            out[kind]["radix"] = R
            out[kind]["executed_real_tflops"] = 8.0 * n ** 3 / R / t / 1e9
        print(json.dumps({kind: {kk: vv for kk, vv in out[kind].items() if kk != "split_phases_ms"}}),
              file=sys.stderr, flush=True)
        del Y, Y64
        torch.cuda.empty_cache()
    line = {"metric": f"Toeplitz/Hankel/DFT/CauchyEig A·C TFLOP/s n={n}, split vs FP64",
            "value": out["toeplitz"]["split_tflops"],
            "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": out["toeplitz"]["split_ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64 (split: bf16 modular slices)", "data": "synthetic",
            "config": {"workload": f"toeplitz/hankel/dft/cauchyeig n=k={n}", "n_moduli": nmod,
                       "l2": "inputs 0.5-1 GiB > L2, no flush"},
            "cublas_dgemm_tflops": dgemm, "kinds": out}
    return line


def fp64_dgemm_rate(dev, stream):
    """cuBLAS DGEMM 8192^3 TFLOP/s on this GPU (best of 3 after one warm-up): the FP64
    tensor-core roofline denominator (MEASURED_PEAKS.json carries no FP64 figure)."""
    import torch
    a = torch.randn(8192, 8192, device=dev, dtype=torch.float64)
    torch.matmul(a, a)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        torch.matmul(a, a)
        e1.record(stream)
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a
    return 2 * 8192 ** 3 / (best * 1e-3) / 1e12


def run_cfg0(args, ws, rank, local, compact=False):
    """Cauchy multiply on the FP64 plain path at n = k = 2048 over seeds 0..4 (A ~ U[-1,1],
    d = sort(U(0,1)), w_j ~ U(d_j, d_j+1), u, v ~ N(0,1)): median of the timed calls per seed
    (CUDA events, after args.warmup), error against the oracle's FP64 A@H, the split path
    beside it, and the FP64 roofline against cuBLAS DGEMM measured in the same run.  e2e: the
    same multiply through the host-pointer entry point (pinned host arrays, copies inside the
    timed region).  CPU baseline: the restatement of PSCAUCHY_COMPUTE on a 2 x 2 grid, block 64
    (4 emulated ranks), and a dense A@H, on all host cores.  Returns the JSON object."""
    import numpy as np
    import torch
    import psmma_git_gb300 as P
    from oracle import psmma_oracle as O
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = 2048
    flops = 2.0 * n ** 3
    stream = torch.cuda.current_stream()
    steps = max(10, args.steps)
    col = lambda x: torch.from_numpy(np.ascontiguousarray(np.asarray(x).T)).to(dev).t()  # noqa: E731
    per_seed = []
    for seed in range(5):
        A = O.cfg_matrix(n, n, seed=seed)
        gen = O.cfg_cauchy_generators(n, seed=seed)
        dA, dg = col(A), col(gen)
        ref = O.dense_product("cauchy", 1.0, A, gen, 0.0, None, n)
        out = {}
        for prec in ["fp64", "split"]:
            dQ = P.fortran_empty(n, n, torch.float64, dev)
            for _ in range(args.warmup):
                P.psmma_cauchy(n, n, 1.0, dA, dg, 0.0, dQ, precision=prec, n_moduli=args.n_moduli, stream=stream)
            torch.cuda.synchronize()
            ts = []
            for _ in range(steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                P.psmma_cauchy(n, n, 1.0, dA, dg, 0.0, dQ, precision=prec, n_moduli=args.n_moduli, stream=stream)
                e1.record(stream)
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            out[prec] = {"ms": float(np.median(ts)), "tflops": flops / (np.median(ts) * 1e-3) / 1e12,
                         "rel_err_vs_oracle": O.rel_fro(dQ.t().contiguous().cpu().numpy().T, ref)}
        per_seed.append(out)
    dgemm = fp64_dgemm_rate(dev, stream)
    # e2e (seed 0): psmma_cauchy_host on pinned host arrays, FP64 path
    A = O.cfg_matrix(n, n, seed=0)
    gen = O.cfg_cauchy_generators(n, seed=0)
    hA = torch.empty((n, n), dtype=torch.float64, pin_memory=True)
    hA.numpy()[:] = A.T
    hG = torch.empty((4, n), dtype=torch.float64, pin_memory=True)
    hG.numpy()[:] = gen.T
    hQ = torch.zeros((n, n), dtype=torch.float64, pin_memory=True)
    nA, nG, nQ = hA.numpy().T, hG.numpy().T, hQ.numpy().T
    for _ in range(args.warmup):
        P.psmma_cauchy(n, n, 1.0, nA, nG, 0.0, nQ)
    t0 = time.perf_counter()
    for _ in range(steps):
        P.psmma_cauchy(n, n, 1.0, nA, nG, 0.0, nQ)
    te = (time.perf_counter() - t0) / steps
    e2e_err = O.rel_fro(np.asarray(nQ), O.dense_product("cauchy", 1.0, A, gen, 0.0, None, n))
    # CPU baseline: the reference's ring on a 2 x 2 grid and a dense A@H (seed 0)
    t0 = time.perf_counter()
    Qr = O.ps_compute("cauchy", n, n, 1.0, A, gen, 0.0, np.zeros((n, n)), nprow=2, npcol=2, nb=64)
    t_ring = time.perf_counter() - t0
    t0 = time.perf_counter()
    dense = O.dense_product("cauchy", 1.0, A, gen, 0.0, None, n)
    t_dense = time.perf_counter() - t0
    fp64 = [s_["fp64"]["tflops"] for s_ in per_seed]
    v = float(np.median(fp64))
    traffic = profile_traffic("fp64_cauchy_n2048")
    line = {"metric": "Cauchy A·H TFLOP/s n=2048, FP64 plain path (cfg0)", "value": v, "unit": "TFLOP/s",
            "n_gpus": 1, "steps": steps, "warmup": args.warmup,
            "ms_per_step": float(np.median([s_["fp64"]["ms"] for s_ in per_seed])), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "psmma_cauchy FP64 n=k=2048, seeds 0..4 (median over seeds of the median "
                                   "over steps)", "n": n, "l2": "inputs 32 MiB < L2: no flush (small case)"},
            "seeds": per_seed,
            "split_tflops_median": float(np.median([s_["split"]["tflops"] for s_ in per_seed])),
            "max_rel_err_vs_oracle": {p: max(s_[p]["rel_err_vs_oracle"] for s_ in per_seed)
                                      for p in ("fp64", "split")},
            "roofline": {"bound": "tensor", "achieved": v, "peak": dgemm, "unit": "TFLOP/s", "frac": v / dgemm,
                         "traffic": traffic, "kernel": "k_struct_f64<KIND_CAUCHY>",
                         "algorithmic_bytes": 16.0 * n * n + 32.0 * n,
                         "peak_source": "cuBLAS DGEMM 8192^3 measured in this run (FP64 tensor-core proxy; "
                                        "MEASURED_PEAKS.json has no FP64 figure)",
                         "traffic_source": "ncu dram__bytes_read+write of one launch (profiles/fp64_dmma_ncu.md)"
                         if traffic else None},
            "e2e": {"value": flops / te / 1e12, "unit": "TFLOP/s", "h2d_bytes_per_step": 8 * n * n + 32 * n,
                    "d2h_bytes_per_step": 8 * n * n, "ms_per_step": te * 1e3, "steps": steps,
                    "api": "psmma_cauchy_host (pinned host buffers), FP64 path", "rel_err_vs_oracle": e2e_err},
            "cpu_baseline": {"value": flops / t_ring / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(),
                             "kind": "port", "sample": f"whole product, ring restatement 2x2 grid nb=64: "
                                                       f"{t_ring:.2f} s; dense A@H: {t_dense:.2f} s"},
            "ring_vs_dense_rel": O.rel_fro(Qr, dense),
            "gpu_launches": 2 * 5 * (steps + args.warmup)}
    return line


def run_redist(args, ws, rank, local):
    """The REDIST copy (PDGEMR2D) of an n x n matrix from the reference tests' layout (2 x 2
    grid, 64 x 64 blocks, Test/psmma_testcauchy.f90:80) to row panels over the 4 ranks, with the
    4 ranks' local arrays on one GPU: the pack kernel of every rank, then the unpack kernel of
    every rank (the all-to-all between them is the caller's and is not timed here; its
    receive buffers are assembled once before timing).  Algorithmic bytes: 16 per element
    (8 read + 8 written) per kernel.  One JSON line."""
    import torch
    from psmma_git_gb300.redist import Grid, RedistPlan, descinit
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    n = args.redist_n
    ga, gb = Grid(2, 2, "R"), Grid(4, 1, "R")
    plans, A, sends, recvs, B = [], [], [], [], []
    g = torch.Generator(device=dev)
    g.manual_seed(3)
    for r in range(4):
        da = descinit(n, n, 64, 64, 0, 0, ga, r)
        db = descinit(n, n, -(-n // 4), n, 0, 0, gb, r)
        p = RedistPlan(n, n, da, ga, db, gb, r)
        plans.append(p)
        a = torch.empty((p.a_shape[1], da[8]), dtype=torch.float64, device=dev).t()
        a.copy_(torch.rand(a.shape, generator=g, device=dev, dtype=torch.float64))
        A.append(a)
        sends.append(torch.empty(sum(p.send_counts), dtype=torch.float64, device=dev))
        B.append(torch.empty((p.b_shape[1], db[8]), dtype=torch.float64, device=dev).t())
    for r in range(4):
        plans[r].pack(A[r], sends[r])
    for r in range(4):  # the exchange, once: rank r's segments from every sender
        parts = []
        for s in range(4):
            d = sum(plans[s].send_counts[:r])
            parts.append(sends[s][d:d + plans[s].send_counts[r]])
        recvs.append(torch.cat(parts))
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        for r in range(4):
            plans[r].pack(A[r], sends[r], stream)
        for r in range(4):
            plans[r].unpack(recvs[r], B[r], stream)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    t_pack = t_unpack = 0.0
    for _ in range(args.steps):
        ev[0].record(stream)
        for r in range(4):
            plans[r].pack(A[r], sends[r], stream)
        ev[1].record(stream)
        for r in range(4):
            plans[r].unpack(recvs[r], B[r], stream)
        ev[2].record(stream)
        torch.cuda.synchronize()
        t_pack += ev[0].elapsed_time(ev[1])
        t_unpack += ev[1].elapsed_time(ev[2])
    t_pack /= args.steps
    t_unpack /= args.steps
    # the round trip must reproduce A: gather the row panels back and compare with a
    # direct construction of the 2x2 layout from the panels' global rows
    rows = [torch.arange(n, device=dev)[torch.arange(n, device=dev) // (-(-n // 4)) == r] for r in range(4)]
    Gm = torch.empty((n, n), dtype=torch.float64, device=dev)
    for r in range(4):
        Gm[rows[r]] = B[r]
    bad = 0
    for r in range(4):
        pr, pc = ga.coords(r)
        ri = torch.arange(n, device=dev)
        rr = ri[(ri // 64) % 2 == pr]
        cc = ri[(ri // 64) % 2 == pc]
        bad += int((Gm[rr][:, cc] != A[r]).sum())
    byts = 16.0 * n * n
    pk = peaks()
    gbs_pack, gbs_unpack = byts / t_pack / 1e6, byts / t_unpack / 1e6
    line = {"metric": f"block-cyclic redistribution (PDGEMR2D pack + unpack) GB/s, n={n}, 2x2 nb=64 -> 4x1 panels",
            "value": 2 * byts / (t_pack + t_unpack) / 1e6, "unit": "GB/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_pack + t_unpack, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"REDIST of an {n} x {n} FP64 matrix, 4 emulated ranks on one GPU",
                       "l2": "2 GiB per pass > L2, no flush"},
            "pack_ms": t_pack, "unpack_ms": t_unpack, "pack_gbs": gbs_pack, "unpack_gbs": gbs_unpack,
            "mismatches": bad, "gpu_launches": 8 * args.steps,
            "roofline": {"bound": "hbm", "achieved": 2 * byts / (t_pack + t_unpack) / 1e6, "peak": pk["hbm"],
                         "unit": "GB/s", "frac": 2 * byts / (t_pack + t_unpack) / 1e6 / pk["hbm"],
                         "traffic": None, "kernel": "k_pack / k_unpack", "peak_source": pk["source"]}}
    print(json.dumps(line), flush=True)
    return 0 if bad == 0 else 1


def run_merge_level(args, ws, rank, local, compact=False):
    """Batched divide-and-conquer merge level: 64 independent Cauchy multiplies Q_i = A_i H_i,
    n_i log-uniform in [256, 8192] (seeded), generators as the n = 2048 workload (d sorted
    uniform, w interlacing, u, v normal), A_i uniform[-1,1] resident in HBM.  The
    off-diagonal blocks of each H_i are compressed at tol 1e-14 by RRQR (the reference's
    Compress_RRQR) and by the structured RRLU; the products run as grouped launches in one
    CUDA graph.  value = dense-equivalent sum(2 n^3) / time (effective), executed flops
    reported beside it.  Rooflines: the grouped modular GEMMs (BF16 flops = executed product
    flops x moduli, against the sustained BF16 peak) and the QR compression (its
    factorisation flops against the in-run DGEMM rate, the FP64 tensor-core proxy; the QR runs
    on the FP64 FMA pipe).  compact: the Cauchy RRQR / RRLU and Toeplitz RRQR runs only, a
    shorter CPU sample.  Returns the JSON object."""
    import numpy as np
    import torch
    import psmma_git_gb300 as P
    from oracle import psmma_oracle as O
    if rank != 0:
        return None
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pk = peaks()
    dgemm = fp64_dgemm_rate(dev, torch.cuda.current_stream())
    sizes = O.cfg_batch_sizes(args.batch_count, 256, 8192, seed=7)
    g = torch.Generator(device=dev)
    g.manual_seed(3)
    probs = []
    for i, n in enumerate(sizes):
        gen = torch.from_numpy(np.ascontiguousarray(O.cfg_cauchy_generators(n, seed=100 + i).T)).to(dev).t()
        A = P.fortran_empty(n, n, torch.float64, dev)
        A.copy_(torch.rand(n, n, generator=g, device=dev, dtype=torch.float64).mul_(2).sub_(1))
        Q = P.fortran_empty(n, n, torch.float64, dev)
        Q.zero_()
        probs.append((A, gen, Q))
    torch.cuda.synchronize()
    eff = sum(2.0 * n ** 3 for n in sizes)
    # dense FP64 references of the smallest problems (accuracy check)
    check = sorted(range(len(sizes)), key=lambda i: sizes[i])[: args.batch_check]
    refs = {}
    for i in check:
        A, gen, _ = probs[i]
        n = sizes[i]
        R = P.fortran_empty(n, n, torch.float64, dev)
        P.psmma_cauchy(n, n, 1.0, A, gen, 0.0, R)
        refs[i] = R
    torch.cuda.synchronize()
    out = {}
    precisions = ["split"] + (["fp64"] if args.merge_fp64 else [])
    # the eigensolver's matrices of the same sizes (psmma_cauchyeig generators, 1% of the roots
    # next to their pole), compressed by RRQR: the natural caller of the merge level
    eig_probs = []
    for i, n in enumerate(sizes):
        F, U, V, dl, dr = O.eig_generators(n, seed=200 + i, tiny=n // 100)
        gen = torch.from_numpy(np.ascontiguousarray(np.stack([F, U, V, dl, dr]))).to(dev).t()
        eig_probs.append((probs[i][0], gen, probs[i][2]))
    # Toeplitz multiplies of the same sizes (PSTOEPLITZ_COMPUTE's low-rank branch, RRQR):
    # H(i, j) = 1 / (j - i + 0.5), numerically low-rank off the diagonal blocks
    toep_probs, toep_refs = [], {}
    for i, n in enumerate(sizes):
        g = torch.from_numpy(1.0 / (np.arange(2 * n - 1) - (n - 1) + 0.5)).to(dev)
        toep_probs.append((probs[i][0], g, P.fortran_empty(n, n, torch.float64, dev)))
    for i in check:
        n = sizes[i]
        R = P.fortran_empty(n, n, torch.float64, dev)
        P.psmma_toeplitz(n, n, 1.0, toep_probs[i][0], toep_probs[i][1], 0.0, R)
        toep_refs[i] = R
    runs = ([(c, p, "cauchy") for c in ["rrqr", "rrlu"] for p in precisions] +
            ([] if compact else [(c, "split", "cauchyeig") for c in ["rrqr", "rrlu"]]) +
            [("rrqr", "split", "toeplitz")])

    def call(batch, kw, kind):
        if kind == "toeplitz":
            return P.toeplitz_batch_lowrank(batch, 1.0, 0.0, tol=kw["tol"], precision=kw["precision"],
                                            n_moduli=kw["n_moduli"])
        return P.cauchy_batch_lowrank(batch, 1.0, 0.0, **kw)

    for comp, prec, kind in runs:
        eig = kind == "cauchyeig"
        batch = eig_probs if eig else toep_probs if kind == "toeplitz" else probs
        kw = dict(compressor=comp, tol=1e-14, precision=prec, n_moduli=args.n_moduli, eig=eig)
        tuned = None
        if prec == "split" and not args.no_tune and kind == "cauchy":
            tkw = {k: v for k, v in kw.items() if k != "eig"}
            tuned = P.tune_batch(probs, 1.0, 0.0, **tkw)  # untimed; later calls use its choice
        for _ in range(args.warmup if prec == "split" else 1):
            ranks, info = call(batch, kw, kind)
        torch.cuda.synchronize()
        steps = args.steps if prec == "split" else 1
        times = []
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record()
            ranks, info = call(batch, kw, kind)
            e1.record()
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        if eig:
            err = None  # checked against the dense product by the tests (no dense eig reference here)
        elif kind == "toeplitz":
            err = max(float(torch.linalg.norm(toep_probs[i][2] - toep_refs[i]) / torch.linalg.norm(toep_refs[i]))
                      for i in check)
        else:
            err = max(float(torch.linalg.norm(probs[i][2] - refs[i]) / torch.linalg.norm(refs[i]))
                      for i in check)
        # per-phase trace of one more call (eager launches, one event per phase)
        lib = P.load()
        lib.psmma_set_profiling(1)
        call(batch, kw, kind)
        torch.cuda.synchronize()
        ms = (C_float * 40)()
        names = (C_charp * 40)()
        m = lib.psmma_profile_read(ms, names, 40)
        lib.psmma_set_profiling(0)
        phases = [[names[j].decode(), round(ms[j], 3)] for j in range(max(0, m))]
        t = statistics.median(times)
        key = f"{comp}_{prec}" + ("_eig" if eig else "_toeplitz" if kind == "toeplitz" else "")
        gemm_ms = sum(v for nm, v in phases if nm.startswith("g_gemm"))
        comp_ms = sum(v for nm, v in phases if nm.startswith("compress"))
        roof = {}
        if prec == "split" and gemm_ms > 0:
            bf = info["executed_flops"] * args.n_moduli
            roof["grouped_gemm"] = {"bound": "tensor", "achieved": bf / (gemm_ms * 1e-3) / 1e12,
                                    "peak": pk["bf16_sustained"], "unit": "TFLOP/s",
                                    "frac": bf / (gemm_ms * 1e-3) / 1e12 / pk["bf16_sustained"],
                                    "traffic": None, "kernel": "k_crt_gemm<*, GroupGemm>",
                                    "flops": bf, "ms": gemm_ms,
                                    "note": "BF16 flops = executed product flops x moduli (K padding not "
                                            f"counted); {pk['source']} cuBLAS bf16 sustained"}
        if comp == "rrqr" and comp_ms > 0:
            roof["qr_compression"] = {"bound": "tensor", "achieved": info["compress_flops"] / (comp_ms * 1e-3) / 1e12,
                                      "peak": dgemm, "unit": "TFLOP/s",
                                      "frac": info["compress_flops"] / (comp_ms * 1e-3) / 1e12 / dgemm,
                                      "traffic": None, "kernel": "k_qr_tiles + k_rrqr_grouped",
                                      "flops": info["compress_flops"], "ms": comp_ms,
                                      "note": "factorisation flops (4 m n (r+1) + 4 m r^2 per block) against "
                                              "the in-run cuBLAS DGEMM rate"}
        out[key] = {
            "ms_per_step": t, "steps": steps, "effective_tflops": eff / t / 1e9,
            "executed_tflops": info["executed_flops"] / t / 1e9,
            "executed_flops": info["executed_flops"], "compress_flops": info["compress_flops"],
            "ranks": {"max": int(max(ranks)), "mean": float(np.mean(ranks)), "min": int(min(ranks))},
            "full_rank_blocks": info["full_rank_blocks"], "rel_err_vs_dense_fp64": err,
            "graph_reused": info.get("graph_reused"),
            "autotune": tuned, "roofline": roof or None, "phases_ms": phases}
        print(json.dumps({key: {kk: vv for kk, vv in out[key].items() if kk != "phases_ms"}}), file=sys.stderr,
              flush=True)
    # CPU baseline: the oracle's restatement of the merge level (Compress_RRQR + DGEMMs) on the
    # smallest problems until ~args.cpu_seconds of work
    cpu = None
    cpu_seconds = min(args.cpu_seconds, 6.0) if compact else args.cpu_seconds
    if not args.no_cpu:
        order = sorted(range(len(sizes)), key=lambda i: sizes[i])
        done_fl, t_cpu, used = 0.0, 0.0, []
        for i in order:
            n = sizes[i]
            A = probs[i][0].cpu().numpy()
            gen = probs[i][1].cpu().numpy()
            t0 = time.perf_counter()
            O.merge_level_product(A, gen, np.zeros((n, n)), 1.0, 0.0, "rrqr", 1e-14)
            t_cpu += time.perf_counter() - t0
            done_fl += 2.0 * n ** 3
            used.append(n)
            if t_cpu > cpu_seconds:
                break
        cpu = {"value": done_fl / t_cpu / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"{len(used)} smallest problems (n = {min(used)}..{max(used)}) of the batch, "
                         "oracle merge level with RRQR, numpy/OpenBLAS threads = cores"}
    head = out["rrqr_split"]
    line = {"metric": "merge level: effective TFLOP/s, sum(2 n^3) / t, "
                      f"{len(sizes)} Cauchy multiplies n log-uniform [256, 8192], off-diagonal blocks RRQR at 1e-14",
            "value": head["effective_tflops"], "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 (split: bf16 modular slices)",
            "data": "synthetic",
            "config": {"workload": "batched merge level", "count": len(sizes), "sum_n": sum(sizes),
                       "n_max": max(sizes), "n_moduli": args.n_moduli, "tol": 1e-14,
                       "l2": "inputs ~ 10 GB > L2, no flush needed"},
            "roofline": head["roofline"]["grouped_gemm"] if head.get("roofline") else None,
            "cublas_dgemm_tflops": dgemm, "compressors": out, "cpu_baseline": cpu}
    return line


import ctypes  # noqa: E402

C_float = ctypes.c_float
C_charp = ctypes.c_char_p


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="psmma", choices=["psmma", "reference"])
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    # 13 moduli: the fewest that meet the metric's <= 1e-12 error on this workload (measured
    # 2.6e-13; 12 moduli lose 7.6 bits of budget)
    ap.add_argument("--n-moduli", type=int, default=13)
    ap.add_argument("--cpu-cols", type=int, default=CPU_COLS)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--serving", action="store_true", help="run the serving-loop sweep instead")
    ap.add_argument("--rates", type=float, nargs="+", default=[5.0, 10.0, 20.0, 40.0])
    ap.add_argument("--inflight", type=int, default=4)
    ap.add_argument("--serve-seconds", type=float, default=6.0)
    ap.add_argument("--serve-nmax", type=int, default=16384)
    ap.add_argument("--serve-budget-gib", type=int, default=96)
    ap.add_argument("--p99-bound-ms", type=float, default=250.0,
                    help="serving: the stated p99 latency bound the sweep is checked against")
    ap.add_argument("--merge-level", action="store_true", help="run the batched merge level (64 problems)")
    ap.add_argument("--cfg1", action="store_true", help="run the Toeplitz/Hankel/DFT multiplies at n = 8192")
    ap.add_argument("--cfg1-n", type=int, default=8192)
    ap.add_argument("--batch-count", type=int, default=64)
    ap.add_argument("--batch-check", type=int, default=8)
    ap.add_argument("--merge-fp64", action="store_true", help="also time the FP64 path of the merge level")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-tune", action="store_true", help="merge level: skip the grouped-GEMM autotuner")
    ap.add_argument("--redist", action="store_true", help="time the block-cyclic redistribution kernels")
    ap.add_argument("--cfg0", action="store_true", help="run the FP64 Cauchy multiply at n = 2048 over 5 seeds")
    ap.add_argument("--redist-n", type=int, default=16384)
    ap.add_argument("--strong", action="store_true",
                    help="with --gpus N: one n x n problem split in N row panels (strong scaling)")
    ap.add_argument("--case", default="", help="profiling case PREC:KIND (e.g. fp64:cauchy) at size --n")
    ap.add_argument("--no-extra", action="store_true",
                    help="default line: skip the compact cfg0 / cfg1 / merge-level / serving entries")
    args = ap.parse_args()
    ws, rank, local = dist_init(args)
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    from psmma_git_gb300 import build as B
    if rank == 0:
        B.build()
    barrier(ws)
    for flag, fn in (("serving", run_serving), ("merge_level", run_merge_level), ("cfg1", run_cfg1),
                     ("cfg0", run_cfg0)):
        if getattr(args, flag):
            line = fn(args, ws, rank, local)
            if line is not None:
                print(json.dumps(line), flush=True)
            return 0
    if args.redist:
        return run_redist(args, ws, rank, local)
    if args.case:
        return run_case(args, ws, rank, local)
    return run_gpu(args, ws, rank, local)


if __name__ == "__main__":
    sys.exit(main())
