"""Benchmark of the contraction hot path on one GB300 (replicas on N GPUs).

Workload (default): the single large pairwise contraction. A has rank 27 and
B rank 25, all index dimensions 2, with 13 shared labels: a complex GEMM of
M = 2^14, N = 2^12, K = 2^13. Both operands' labels are seeded-randomly
permuted, so both need a transpose. Entries are complex64 with real and
imaginary parts i.i.d. N(0, 1/2), scaled by 2^-10 (synthetic, seeded).

One step = Tensor::ContractTensors on the device in a split-precision
tensor-core form: permute+split A, permute+split B, tcgen05 product. The
TF32x3, BF16x3 and FP16x3 forms are all timed; the headline is the fastest
whose error on the step is within 1e-5 of complex128. Metric: effective
TFLOP/s = 4 x PathInfo flops / step time = 8 M N K / t. Inputs (1.34 GB) are
larger than L2 (129 MB), so no flush is needed between steps.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

`--impl reference` times the reference's CPU algorithm (the oracle port:
DefaultPermuter restated in C with OpenMP plus OpenBLAS cgemm through numpy)
on a bounded sample of the same contraction (s common labels fixed, so the
transposes and the GEMM shrink by the same factor).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

N_LEFT, N_COMMON, N_RIGHT = 14, 13, 12
SEED = 20240601
METRIC = "slices/s & eff. TFLOP/s: TC-split vs plain FP32 on GB300 at ≤1e-5 rel err"


def _perm(seed, r):
    return [int(i) for i in np.random.default_rng(seed).permutation(r)]


def workload(n_left=N_LEFT, n_common=N_COMMON, n_right=N_RIGHT):
    """Labels, shapes and the axis orders ContractTensors derives from them."""
    left = ["l%d" % i for i in range(n_left)]
    common = ["c%d" % i for i in range(n_common)]
    right = ["r%d" % i for i in range(n_right)]
    a_lab = [(left + common)[i] for i in _perm(SEED, n_left + n_common)]
    b_lab = [(common + right)[i] for i in _perm(SEED + 1, n_common + n_right)]
    # Tensor::ContractTensors label algebra: left = A\B, common = A∩B (A order).
    lft = [x for x in a_lab if x not in b_lab]
    rgt = [x for x in b_lab if x not in a_lab]
    com = [x for x in a_lab if x in b_lab]
    a_perm = [a_lab.index(x) for x in lft + com]            # A -> (left, common)
    b_perm_kn = [b_lab.index(x) for x in com + rgt]         # B -> (common, right)
    b_perm_nk = [b_lab.index(x) for x in rgt + com]         # B -> (right, common)
    return dict(a_lab=a_lab, b_lab=b_lab, a_shape=[2] * len(a_lab), b_shape=[2] * len(b_lab),
                a_perm=a_perm, b_perm_kn=b_perm_kn, b_perm_nk=b_perm_nk,
                m=2 ** n_left, n=2 ** n_right, k=2 ** n_common)


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.tmp = None

    def __enter__(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.tmp is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.tmp.flush()
        rows = []
        with open(self.tmp.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.tmp.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = []
        for i, nm in enumerate(names):
            if any(r[5 + i].lower().startswith("active") for r in rows):
                reasons.append(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def measured_peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def _cpu_case(s_common):
    """Inputs of the config-1 contraction with s_common shared labels fixed
    (the transposes and the GEMM shrink by the same factor 2^s_common)."""
    import numpy as np

    w = workload(N_LEFT, N_COMMON - s_common, N_RIGHT)
    rng = np.random.default_rng(SEED)
    na, nb = 2 ** len(w["a_lab"]), 2 ** len(w["b_lab"])
    a = ((rng.standard_normal(na) + 1j * rng.standard_normal(na)) * np.sqrt(0.5) * 2**-10).astype(np.complex64)
    b = ((rng.standard_normal(nb) + 1j * rng.standard_normal(nb)) * np.sqrt(0.5) * 2**-10).astype(np.complex64)
    return w, a, b


def _cpu_step(w, a, b, nthreads=0):
    from oracle import port

    t0 = time.perf_counter()
    port.contract(a, w["a_shape"], w["a_perm"], b, w["b_shape"], w["b_perm_kn"], w["m"], w["n"],
                  w["k"], nthreads)
    return time.perf_counter() - t0


def _cpu_sample_text(s_common, runs, t):
    return ("config-1 contraction with %d of 13 shared labels fixed (M=2^14, N=2^12, K=2^%d), "
            "median of %d runs, %.2f s each" % (s_common, N_COMMON - s_common, runs, t))


def cpu_sample(nthreads=0, s_common=1, reps=3):
    """The oracle port on the config with s_common shared labels fixed."""
    from oracle import port

    w, a, b = _cpu_case(s_common)
    _cpu_step(w, a, b, nthreads)  # warm-up
    t = statistics.median(_cpu_step(w, a, b, nthreads) for _ in range(reps))
    flops = 8.0 * w["m"] * w["n"] * w["k"]
    return {"value": flops / t / 1e12, "unit": "TFLOP/s", "cores": port.max_threads(),
            "kind": "port", "sample": _cpu_sample_text(s_common, reps, t)}


def run_reference(args, rank, world):
    """The reference's CPU arithmetic for the path (the oracle port: the
    reference's permute + row-major CBLAS cgemm on all host cores) on a
    bounded sample of config 1: W warm-up and K timed steps, each step one
    contraction with 2 of the 13 shared labels fixed."""
    if rank != 0:
        return
    from oracle import port

    s_common = 2
    w, a, b = _cpu_case(s_common)
    for _ in range(args.warmup):
        _cpu_step(w, a, b)
    times = [_cpu_step(w, a, b) for _ in range(args.steps)]
    t = statistics.median(times)
    value = 8.0 * w["m"] * w["n"] * w["k"] / t / 1e12
    info = {"value": value, "unit": "TFLOP/s", "cores": port.max_threads(), "kind": "port",
            "sample": _cpu_sample_text(s_common, args.steps, t)}
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "TFLOP/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64 (fp32)", "data": "synthetic",
            "config": {"workload": "config 1: rank-27 x rank-25 contraction, 13 shared labels "
                                   "(M=2^14, N=2^12, K=2^13), complex64",
                       "sample": info["sample"]},
            "cpu_baseline": info,
            "e2e": {"value": value, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def apply_tc_knobs(args):
    """The tensor-core product settings given on the command line."""
    import jet_gb300.capi as capi

    if args.tc_variant is not None:
        capi.set_tc_variant(args.tc_variant)
    if args.tc_chunk is not None:
        capi.set_tc_chunk_depth(args.tc_chunk)
    if args.tc_persistent is not None:
        capi.set_tc_persistent(args.tc_persistent)


def run_ours(args, rank, world, local_rank):
    import torch

    import jet_gb300.capi as capi

    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    apply_tc_knobs(args)
    w = workload(12, N_COMMON, 12) if args.small else workload()
    m, n, k = w["m"], w["n"], w["k"]
    kp = k
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + rank)
    # torch.randn on complex draws re, im i.i.d. N(0, 1/2).
    A = torch.randn(m * k, dtype=torch.complex64, device=dev, generator=g) * 2.0**-10
    B = torch.randn(k * n, dtype=torch.complex64, device=dev, generator=g) * 2.0**-10
    C = torch.empty(m * n, dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream(dev)
    flops = 8.0 * m * n * k  # = 4 x PathInfo flops (size(C) * 2 * K)

    # Accuracy of a step's C against complex128 on 32 rows.
    rows = 32
    At = capi.permute(A, w["a_shape"], w["a_perm"]).view(m, k)[:rows].cpu().numpy()
    Bt = capi.permute(B, w["b_shape"], w["b_perm_kn"]).view(k, n).cpu().numpy()
    ref_rows = At.astype(np.complex128) @ Bt.astype(np.complex128)
    del At, Bt

    def rel_err_of(c):
        got = c.view(m, n)[:rows].cpu().numpy()
        return float(np.linalg.norm(got - ref_rows) / np.linalg.norm(ref_rows))

    def run_form(form):
        """Times `args.steps` steps of split A, split B, split product (forms
        ending in _3m: the 3M product on six planes per operand)."""
        base, _, algo = form.partition("_")
        three_m = algo == "3m"
        bf, hf = base == "bf16x3", base == "fp16x3"
        # --tc-variant 1: the N = 256 main loop (six B planes with -im).
        wide = (bf or hf) and not three_m and args.tc_variant == 1
        fmt = capi.FMT_BF16 if bf else capi.FMT_FP16 if hf else capi.FMT_TF32
        word = torch.int16 if (bf or hf) else torch.float32
        aplanes = 6 if three_m else 4
        bplanes = 6 if (three_m or wide) else 4 if (bf or hf) else capi.tc_b_planes()
        extra_a = capi.SPLIT_SUM if three_m else 0
        extra_b = capi.SPLIT_SUM if three_m else capi.SPLIT_NEG_IM if wide else 0
        pa = torch.empty(aplanes * m * kp, dtype=word, device=dev)
        pb = torch.empty(bplanes * n * kp, dtype=word, device=dev)
        e2 = torch.empty(2, dtype=torch.int32, device=dev)  # FP16: max exponents of A, B

        def step16(events=None):
            """16-bit forms: the general split and product stages."""
            if events:
                events[0].record(stream)
            if hf:
                capi.max_exponent(A, stream=stream, out=e2[0:1])
            capi.split_planes(A, w["a_shape"], w["a_perm"], m, k, kp, pa, fmt, extra=extra_a,
                              e_max=e2[0:1] if hf else None, stream=stream)
            if events:
                events[1].record(stream)
            if hf:
                capi.max_exponent(B, stream=stream, out=e2[1:2])
            capi.split_planes(B, w["b_shape"], w["b_perm_nk"], n, k, kp, pb, fmt, extra=extra_b,
                              e_max=e2[1:2] if hf else None, stream=stream)
            if events:
                events[2].record(stream)
            capi.gemm_split(pa, pb, m, n, k, kp, C, fmt,
                            algo=capi.ALGO_3M if three_m else capi.ALGO_4M,
                            e_max2=e2 if hf else None, stream=stream, variant=1 if wide else 0)
            if events:
                events[3].record(stream)

        def step(events=None):
            if bf or hf:
                return step16(events)
            # TF32: the TF32x3 stage entry points (B planes per jetgpu_tc_b_planes).
            if events:
                events[0].record(stream)
            capi.split_tf32(A, w["a_shape"], w["a_perm"], m, k, kp, pa, stream=stream)
            if events:
                events[1].record(stream)
            capi.split_tf32(B, w["b_shape"], w["b_perm_nk"], n, k, kp, pb, n_planes=bplanes,
                            stream=stream)
            if events:
                events[2].record(stream)
            capi.gemm_tf32x3(pa, pb, m, n, k, kp, C, stream=stream)
            if events:
                events[3].record(stream)

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize(dev)
        if capi.take_device_status() != 0:
            raise RuntimeError("device status reports a timeout in the warm-up")
        evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)]
               for _ in range(args.steps)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        with Clocks(local_rank) as clk:
            t0 = time.perf_counter()
            for s in range(args.steps):
                step(evs[s])
            torch.cuda.synchronize(dev)
            wall = time.perf_counter() - t0
        if world > 1:
            torch.distributed.barrier()
        ms_step = evs[0][0].elapsed_time(evs[-1][3]) / args.steps
        if world > 1:
            t = torch.tensor([ms_step], dtype=torch.float64, device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms_step = float(t.item())
        out = {"ms_per_step": ms_step, "value": world * flops / (ms_step * 1e-3) / 1e12,
               "rel_err_vs_fp64": rel_err_of(C),
               "stages_ms": {"split_a": statistics.mean(e[0].elapsed_time(e[1]) for e in evs),
                             "split_b": statistics.mean(e[1].elapsed_time(e[2]) for e in evs),
                             "gemm": statistics.mean(e[2].elapsed_time(e[3]) for e in evs)},
               "clocks": clk.summary(), "wall_s_timed": wall}
        del pa, pb
        return out

    forms = (["tf32x3", "bf16x3", "fp16x3", "bf16x3_3m", "fp16x3_3m"] if args.form == "auto"
             else [args.form])
    results = {f: run_form(f) for f in forms}
    if args.form == "auto":
        # The fastest form whose error on this step meets the 1e-5 bound
        # (TF32x3 if none does).
        ok = [f for f in forms if results[f]["rel_err_vs_fp64"] <= 1e-5] or ["tf32x3"]
        head = min(ok, key=lambda f: results[f]["ms_per_step"])
    else:
        head = args.form
    hr = results[head]
    if args.kernels_only:
        if rank == 0:
            print(json.dumps({"head": head, "forms": results, "m": m, "n": n, "k": k}),
                  flush=True)
        return
    ms_step, value, rel_err = hr["ms_per_step"], hr["value"], hr["rel_err_vs_fp64"]
    clocks, wall = hr["clocks"], hr["wall_s_timed"]
    head_base, _, head_algo = head.partition("_")
    head_prec = {"tf32x3": capi.PREC_TF32X3, "bf16x3": capi.PREC_BF16X3,
                 "fp16x3": capi.PREC_FP16X3}[head_base]
    head_algo = capi.ALGO_3M if head_algo == "3m" else capi.ALGO_4M

    # Plain FP32 form of the same step (permute + SIMT complex GEMM), 2 runs.
    ws_need = capi.contract_workspace_size(w["a_shape"], w["a_perm"], w["b_shape"],
                                           w["b_perm_kn"], m, n, k, capi.C64, capi.PREC_FP32)
    ws = torch.empty(ws_need, dtype=torch.uint8, device=dev)
    C2 = torch.empty_like(C)
    capi.contract(A, w["a_shape"], w["a_perm"], B, w["b_shape"], w["b_perm_kn"], m, n, k,
                  precision=capi.PREC_FP32, out=C2, workspace=ws, stream=stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(2):
        capi.contract(A, w["a_shape"], w["a_perm"], B, w["b_shape"], w["b_perm_kn"], m, n, k,
                      precision=capi.PREC_FP32, out=C2, workspace=ws, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    plain_ms = e0.elapsed_time(e1) / 2
    plain_err = rel_err_of(C2)
    del ws, C2

    # The plain permute of A alone (bitperm_kernel, 2^27 complex64 elements:
    # 1.07 GB read + 1.07 GB written), the transpose of Tensor::Transpose.
    At = torch.empty_like(A)
    capi.permute(A, w["a_shape"], w["a_perm"], out=At, stream=stream)
    e0.record(stream)
    for _ in range(5):
        capi.permute(A, w["a_shape"], w["a_perm"], out=At, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    permute_ms = e0.elapsed_time(e1) / 5
    permute_gbs = 16.0 * A.numel() / (permute_ms * 1e-3) / 1e9
    del At

    # End to end through the public API with host buffers: every step copies
    # its A and B from pinned host memory to the device, contracts them with
    # jetgpu_contract (the headline form) and copies C back to pinned host
    # memory. Steps are pipelined over three device buffer sets, so step i's
    # uploads and the downloads of earlier steps (copy streams) overlap the
    # contractions before it; the host link (about 210 GB/s up, 190 down, 280
    # both ways at once on this machine) moves 1.88 GB per step.
    hA = A.cpu().pin_memory()
    hB = B.cpu().pin_memory()
    n_slots = 3
    slots = [dict(a=torch.empty_like(A), b=torch.empty_like(B), c=torch.empty_like(C),
                  hc=torch.empty(C.shape, dtype=C.dtype).pin_memory()) for _ in range(n_slots)]
    ws_tc = torch.empty(capi.contract_workspace_size(w["a_shape"], w["a_perm"], w["b_shape"],
                                                     w["b_perm_kn"], m, n, k, capi.C64,
                                                     head_prec, head_algo),
                        dtype=torch.uint8, device=dev)
    cs_in = torch.cuda.Stream(dev)
    cs_out = torch.cuda.Stream(dev)
    ev = {key: [torch.cuda.Event() for _ in range(n_slots)] for key in ("in", "comp", "out")}
    for key in ev:
        for e in ev[key]:
            e.record(stream)

    def e2e_step(i):
        j = i % n_slots
        sl = slots[j]
        with torch.cuda.stream(cs_in):
            cs_in.wait_event(ev["comp"][j])       # slot j's inputs consumed by step i-3
            sl["a"].copy_(hA, non_blocking=True)
            sl["b"].copy_(hB, non_blocking=True)
            ev["in"][j].record(cs_in)
        stream.wait_event(ev["in"][j])
        stream.wait_event(ev["out"][j])           # slot j's C read back by step i-3
        capi.contract(sl["a"], w["a_shape"], w["a_perm"], sl["b"], w["b_shape"], w["b_perm_kn"],
                      m, n, k, precision=head_prec, out=sl["c"], workspace=ws_tc,
                      stream=stream, algo=head_algo)
        ev["comp"][j].record(stream)
        with torch.cuda.stream(cs_out):
            cs_out.wait_event(ev["comp"][j])
            sl["hc"].copy_(sl["c"], non_blocking=True)
            ev["out"][j].record(cs_out)

    for i in range(max(2, min(args.warmup, 4))):
        e2e_step(i)
    torch.cuda.synchronize(dev)
    e2e_steps = max(4, args.steps)
    e0.record(stream)
    for i in range(e2e_steps):
        e2e_step(i)
    stream.wait_stream(cs_out)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    e2e_value = world * flops / (e2e_ms * 1e-3) / 1e12
    e2e_err = rel_err_of(slots[(e2e_steps - 1) % n_slots]["hc"])
    del slots, ws_tc

    hbm_peak, bf16_peak, peak_src = measured_peaks()
    # Dense tensor rate of the headline form's operand type: BF16 = measured
    # bf16, TF32 = half of it.
    tf32 = head_base == "tf32x3"
    three_m = head_algo == capi.ALGO_3M
    tc_peak = bf16_peak / 2.0 if tf32 else bf16_peak
    gemm_ms = hr["stages_ms"]["gemm"]
    split_ms = hr["stages_ms"]["split_a"]
    # A per element: read 8 B, write 4 planes (3M: 6) x (2 B BF16 / FP16 |
    # 4 B TF32); FP16 also reads A once more for its max exponent.
    planes = 6 if three_m else 4
    word = 4.0 if tf32 else 2.0
    split_bytes = (8.0 + planes * word + (8.0 if head_base == "fp16x3" else 0.0)) * m * k
    achieved = flops / (gemm_ms * 1e-3) / 1e12
    # DRAM bytes (read + write) per launch of the product at this size: a
    # constant taken from one ncu capture of this workload, not measured in
    # this run (CUDA events cannot count DRAM bytes); null where none was taken.
    traffic = {"tf32x3": 14.77e9, "bf16x3": 7.67e9}.get(head)
    form_names = {"tf32x3": "TF32x3 4M (tcgen05 kind::tf32, hi/lo split, 3 products)",
                  "bf16x3": "BF16x3 4M (tcgen05 kind::f16 on BF16, hi/lo split, 3 products)",
                  "fp16x3": "FP16x3 4M (tcgen05 kind::f16 on FP16 hi/lo of power-of-two "
                            "scaled operands, 3 products)",
                  "bf16x3_3m": "BF16x3 3M (Gauss: 3 real products, each hi/lo split "
                               "3 products, kind::f16 on BF16)",
                  "fp16x3_3m": "FP16x3 3M (Gauss: 3 real products, each hi/lo split "
                               "3 products, kind::f16 on scaled FP16)",
                  "tf32x3_3m": "TF32x3 3M (Gauss: 3 real products, kind::tf32)"}
    kernel_v = {("tf32x3", False): 0, ("bf16x3", False): 2, ("fp16x3", False): 4,
                ("tf32x3", True): 5, ("bf16x3", True): 6, ("fp16x3", True): 7}[(head_base,
                                                                                 three_m)]
    # Tensor-pipe flops per algorithmic flop: 3 split products of each real
    # product; 3M does 3 real products where the algorithmic count has 4.
    pipe_factor = 3.0 * (0.75 if three_m else 1.0)
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "c64 (fp32 data, split-precision tensor-core products, fp32 accumulate)",
        "data": "synthetic (seeded N(0,1/2) * 2^-10 complex64)",
        "config": {"workload": "config 1: rank-27 x rank-25 contraction, 13 shared labels, "
                               "seeded label permutations (M=2^14, N=2^12, K=2^13)",
                   "form": form_names[head], "l2": "inputs 1.34 GB > L2, no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "rel_err_vs_fp64": rel_err,
        "stages_ms": hr["stages_ms"],
        "forms": {f: {"value": r["value"], "ms_per_step": r["ms_per_step"],
                      "rel_err_vs_fp64": r["rel_err_vs_fp64"], "stages_ms": r["stages_ms"]}
                  for f, r in results.items()},
        "plain_fp32": {"ms_per_step": plain_ms,
                       "value": world * flops / (plain_ms * 1e-3) / 1e12,
                       "rel_err_vs_fp64": plain_err},
        "roofline": {"bound": "tensor",
                     "kernel": "tc_gemm_split_kernel<%d>" % kernel_v,
                     "achieved": achieved, "peak": tc_peak, "unit": "TFLOP/s",
                     "frac": achieved / tc_peak,
                     "tensor_pipe_frac": pipe_factor * achieved / tc_peak,
                     "peak_source": ("%s bf16 (%.0f TFLOP/s)" % (peak_src, bf16_peak))
                     if not tf32 else
                     ("TF32 dense = 1/2 of %s bf16 (%.0f TFLOP/s)" % (peak_src, bf16_peak)),
                     "traffic": traffic,
                     "traffic_source": ("constant from one ncu capture of this workload "
                                        "(dram__bytes_read.sum + dram__bytes_write.sum), not "
                                        "measured in this run") if traffic else
                                       "no ncu capture of this form's product at this size",
                     "traffic_algorithmic": planes * word * (m + n) * k + 8.0 * m * n},
        "roofline_split": {"bound": "hbm",
                           "kernel": "max_exp_kernel + bitperm_kernel (split store)"
                           if head_base == "fp16x3" else "bitperm_kernel (split store)",
                           "achieved": split_bytes / (split_ms * 1e-3) / 1e9, "peak": hbm_peak,
                           "unit": "GB/s",
                           "frac": split_bytes / (split_ms * 1e-3) / 1e9 / hbm_peak,
                           "peak_source": peak_src},
        "roofline_permute": {"bound": "hbm", "kernel": "bitperm_kernel (plain store)",
                             "achieved": permute_gbs, "peak": hbm_peak, "unit": "GB/s",
                             "frac": permute_gbs / hbm_peak, "ms": permute_ms,
                             "peak_source": peak_src},
        "e2e": {"value": e2e_value, "unit": "TFLOP/s",
                "h2d_bytes_per_step": int(A.numel() * 8 + B.numel() * 8),
                "d2h_bytes_per_step": int(C.numel() * 8), "ms_per_step": e2e_ms,
                "rel_err_vs_fp64": e2e_err,
                "pipeline": "three device buffer sets; H2D and D2H on copy streams overlap "
                            "the contractions"},
        # per step: 2 splits + 1 product (FP16: + one max-exponent kernel per
        # operand, each after a 4-byte memset)
        "gpu_launches": (5 if head_base == "fp16x3" else 3) * args.steps,
        "wall_s_timed": wall,
        "clocks": clocks,
    }
    if not args.no_sliced and world == 1:
        line["sliced"] = {"config4": run_sliced_leg("config4", batch=16, chunks=2),
                          "config2": run_sliced_leg("config2", batch=2, chunks=2),
                          "m12": m12_leg(batch=8, chunks=4)[0]}
    if rank == 0 and not args.no_cpu_baseline:
        try:
            line["cpu_baseline"] = cpu_sample()
        except Exception as e:  # the baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "error": str(e)}
    if rank == 0:
        print(json.dumps(line), flush=True)


SLICED_CONFIGS = {
    # name: (rows, cols, cycles, removed sites, sliced bonds (config 4: the
    #        fewest), slices per batch, chunks timed, path restarts)
    "2": (7, 7, 14, (), 12, 2, 2, 48),
    "4": (6, 9, 12, (5,), 6, 64, 2, 48),
    "0": (4, 4, 8, (), 0, 1, 1, 8),
    # qutrit variant of config 4: 5x5 sites of dimension 3, 8 layers of Haar
    # unitaries (cycles = layers), 4 sliced bonds -> 81 slices
    "4q": (5, 5, 8, (), 4, 9, 9, 16),
}
QUDIT_DIM = {"4q": 3}
# Configs sliced until a chunk of their slices per batch fits this much HBM
# (the contractor's own plan: arena, workspace, slice-independent buffers).
MEMORY_BUDGET = {"4": 120e9}


def time_sliced_form(jet, tn, path, sliced, prec, batch, chunks, start=None, after=None):
    """Slices/s of one form through Jet::SlicedContractor: one eager warm-up
    chunk (prefix, tuning, graph capture), then `chunks` chunks of `batch`
    slices replayed from the captured graph, timed on the host around the
    synchronous Contract call (it returns the FP64 sum read back from the
    device); runs under 0.2 s are repeated and the median kept."""
    import torch

    sc = jet.SlicedContractorC64(tn, path, sliced, prec)
    sc.set_batch_size(batch)
    n_all = sc.num_slices
    sc.contract(0, batch)
    count = min(n_all, batch * chunks)
    if start is None:
        start = 0 if count == n_all else batch
    if start + count > n_all:
        start = 0
    torch.cuda.synchronize()
    reps = []
    amp = None
    while not reps or sum(reps) < 0.2:
        t1 = time.perf_counter()
        amp = sc.contract(start, count)[0]
        reps.append(time.perf_counter() - t1)
    dt = statistics.median(reps)
    # The first timed chunk's FP64 sum, so that forms timed over different
    # numbers of chunks can be compared on the same slices.
    first_amp = amp if count == batch else sc.contract(start, batch)[0]
    if after is not None:
        after(sc, start)
    out = {"slices_per_s": count / dt, "s_per_slice": dt / count,
           "eff_tflops": 4.0 * sc.slice_dependent_flops * count / dt / 1e12,
           "slices_timed": count, "first_slice": start, "runs": len(reps),
           "arena_gb": sc.arena_bytes / 1e9}
    info = {"amp": amp, "first_chunk_amp": first_amp, "slice_flops": sc.slice_flops,
            "slice_dependent_flops": sc.slice_dependent_flops, "num_slices": n_all}
    del sc
    return out, info


def config_golden(name):
    """The record of a sliced circuit in the golden fixtures (made on the CPU
    by tests/golden/make_network_fixtures.py): circuit, path, sliced bonds
    and, where the oracle could run one, complex128 amplitudes of slices."""
    with open(os.path.join(REPO, "tests", "golden", "network_amplitudes.json")) as f:
        return json.load(f)[name]


def run_sliced_leg(name, batch, chunks, fp32_chunks=1):
    """A sliced circuit of the golden fixtures beside the config-1 line, in
    the tensor-core AUTO form and in plain FP32: slices/s of each and their
    ratio (the target is at least 3x), and each form's error on single
    slices against the complex128 oracle amplitudes of the fixture where it
    has them (config 4), else AUTO's difference from FP32 (config 2)."""
    import jet_gb300 as jet
    from jet_gb300 import capi, circuits

    ent = config_golden(name)
    net = circuits.random_circuit_network(ent["rows"], ent["cols"], ent["cycles"],
                                          seed=ent["seed"], removed=tuple(ent["removed"]))
    path = [tuple(p) for p in ent["path"]]
    sliced = ent["sliced"]
    tn = jet.TensorNetwork(dtype="complex64")
    for lab, sh, d in net.tensors:
        tn.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype="complex64"))
    capi.set_auto_form(capi.PREC_FP16X3)
    forms, errs, amps = {}, {}, {}
    for fname, prec, ch in (("auto", jet.PREC_AUTO, chunks),
                            ("fp32", jet.PREC_FP32, fp32_chunks)):
        forms[fname], info = time_sliced_form(jet, tn, path, sliced, prec, batch, ch)
        amps[fname] = info["first_chunk_amp"]
        if not ent["slices"]:
            continue
        one = jet.SlicedContractorC64(tn, path, sliced, prec)
        one.set_batch_size(1)
        errs[fname] = {}
        for v, rec in ent["slices"].items():
            got = one.contract(int(v), 1)[0]
            want = complex(*rec["oracle_c128"])
            errs[fname]["slice_%s" % v] = abs(got - want) / abs(want)
        del one
    for fname in errs:
        forms[fname]["rel_err_vs_fp64"] = max(errs[fname].values())
        forms[fname]["rel_err_per_slice"] = errs[fname]
    n_q = ent["rows"] * ent["cols"] - len(ent["removed"])
    out = {"workload": "config %s: %dx%d grid%s, %d cycles, %d qubits, %d sliced bonds "
                       "(%d slices), greedy path of %d steps, %d slices per batch"
                       % (name[-1], ent["rows"], ent["cols"],
                          " minus site %d" % ent["removed"][0] if ent["removed"] else "",
                          ent["cycles"], n_q, len(sliced), info["num_slices"], len(path), batch),
           "unit": "slices/s", "slice_pathinfo_flops": info["slice_flops"],
           "forms": forms,
           "tc_vs_plain_speedup": forms["auto"]["slices_per_s"] / forms["fp32"]["slices_per_s"],
           "timing": "host clock around each synchronous chunk replay (graph launch + FP64 "
                     "read-back); warm-up chunk excluded"}
    if errs:
        out["error_reference"] = ("complex128 oracle amplitudes of slices %s (golden fixture)"
                                  % ", ".join(sorted(ent["slices"], key=int)))
    else:
        out["rel_diff_auto_vs_fp32"] = (abs(amps["auto"] - amps["fp32"]) /
                                        max(abs(amps["fp32"]), 1e-300))
        out["error_reference"] = ("none on the CPU (one slice is 3.6e13 PathInfo flops); "
                                  "AUTO's difference from plain FP32 on the first timed chunk")
    return out


def shared_flop_fraction(net, path, sliced, varying):
    """PathInfo flops of the steps that depend neither on the leaves in
    `varying` nor on a sliced bond, as a fraction of one slice's flops: the
    work one run shares across the leaves' alternatives and the slices."""
    dims = dict(net.index_dims())
    for x in sliced:
        dims[x] = 1
    sl = set(sliced)
    nodes = {i: (list(l), i in varying or any(x in sl for x in l))
             for i, (l, _, _) in enumerate(net.tensors)}
    nid = len(nodes)
    total = shared = 0.0
    for a, b in path:
        la, va = nodes.pop(a)
        lb, vb = nodes.pop(b)
        out = [x for x in la if x not in lb] + [x for x in lb if x not in la]
        fl = 2.0 * math.prod(dims[x] for x in out) * math.prod(dims[x] for x in la if x in lb)
        total += fl
        if not (va or vb):
            shared += fl
        nodes[nid] = (out, va or vb)
        nid += 1
    return shared / total


def run_bitstrings(args, jet, net, path, sliced, rows, cols, cycles, removed):
    """The second pass of config 2: seeded-uniform output bitstrings as
    alternatives of the output-cap leaves ("$b"), so that one run yields
    several bitstrings' amplitudes and computes every bitstring-independent
    intermediate once. Timed on a sample (bitstrings per run x slices per
    batch x chunks), reported as bitstring-slices/s with the extrapolated
    time for all bitstrings and slices; the amplitudes of the sample's
    first chunk are checked against separate single-bitstring runs."""
    from jet_gb300 import circuits

    n_q = rows * cols - len(removed)
    n_t = len(net.tensors)
    cap_ids = list(range(n_t - n_q, n_t))  # output caps close the network, one per qubit
    bits = np.random.default_rng(SEED + 1).integers(0, 2, size=(args.bitstrings, n_q))
    nb = args.bitstring_chunk
    batch = args.sliced_batch or 1
    tn = jet.TensorNetwork(dtype="complex64")
    for lab, sh, d in net.tensors:
        tn.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype="complex64"))

    def contractor(chunk_bits):
        sc = jet.SlicedContractorC64(tn, path, sliced, jet.PREC_AUTO)
        sc.set_batch_size(batch)
        for q, node in enumerate(cap_ids):
            vals = []
            for b in chunk_bits:
                vals += [1, 0] if b[q] == 0 else [0, 1]
            sc.set_leaf_alternatives(node, vals, len(chunk_bits))
        return sc

    sc = contractor(bits[:nb])
    sc.contract(0, batch)  # warm-up: prefix, tuning, capture
    count = batch * max(1, args.sliced_chunks or 1)
    reps = []
    while not reps or sum(reps) < 0.2:
        t1 = time.perf_counter()
        amps = sc.contract(batch, count)
        reps.append(time.perf_counter() - t1)
    dt = statistics.median(reps)
    arena = sc.arena_bytes
    del sc
    # Consistency: each bitstring of the chunk contracted on its own.
    worst = 0.0
    for i in range(min(nb, 2)):
        net_b = circuits.random_circuit_network(rows, cols, cycles, seed=SEED, removed=removed,
                                                bitstring=bits[i])
        tb = jet.TensorNetwork(dtype="complex64")
        for lab, sh, d in net_b.tensors:
            tb.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype="complex64"))
        one = jet.SlicedContractorC64(tb, path, sliced, jet.PREC_AUTO)
        one.set_batch_size(batch)
        want = one.contract(batch, count)[0]
        del one
        worst = max(worst, abs(amps[i] - want) / max(abs(want), 1e-300))
    rate = nb * count / dt
    n_slices = 2 ** len(sliced)
    return {"bitstrings": args.bitstrings, "bitstrings_per_run": nb, "slices_per_batch": batch,
            "slices_timed": count, "bitstring_slices_per_s": rate,
            "extrapolated_all_s": args.bitstrings * n_slices / rate,
            "arena_gb": arena / 1e9,
            "shared_flop_fraction": shared_flop_fraction(net, path, sliced, set(cap_ids)),
            "rel_diff_vs_single_bitstring_runs": worst,
            "sharing": "every intermediate that depends on no output cap (and the "
                       "slice-independent prefix) is computed once per run for all its "
                       "bitstrings"}


def run_sliced(args, rank, world, local_rank):
    """Sliced random-circuit amplitudes through Jet::SlicedContractor: every
    slice of a seeded circuit network along one greedy path, in batched
    launches replayed from one CUDA graph, FP64 slice sum. Reports slices/s
    and effective TFLOP/s (4 x PathInfo flops per slice) for AUTO (FP16x3 on
    the large steps; auto_tf32: TF32x3 there), TUNED (the autotuner's fastest
    form per step, tuned on the warm-up chunk), BF16x3 and plain FP32, each
    with its amplitude error against complex128 under --check-fp64."""
    import torch

    import jet_gb300 as jet
    from jet_gb300 import capi, circuits

    torch.cuda.set_device(local_rank)
    apply_tc_knobs(args)
    rows, cols, cycles, removed, n_sliced, batch, chunks, restarts = SLICED_CONFIGS[args.config]
    if args.sliced_batch:
        batch = args.sliced_batch
    if args.sliced_chunks:
        chunks = args.sliced_chunks
    t0 = time.perf_counter()
    qd = QUDIT_DIM.get(args.config, 2)
    if qd != 2:
        net = circuits.qudit_circuit_network(rows, cols, cycles, d=qd, seed=SEED)
    else:
        net = circuits.random_circuit_network(rows, cols, cycles, seed=SEED, removed=removed)
    path = circuits.best_gain_path(net, restarts)
    tn = jet.TensorNetwork(dtype="complex64")
    for lab, sh, d in net.tensors:
        tn.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype="complex64"))
    budget = None
    if args.config in MEMORY_BUDGET and not args.sliced_batch:
        from jet_gb300 import slicing

        # The bonds for both the tensor-core and the plain form's plans.
        cap = MEMORY_BUDGET[args.config]
        sliced, need, batch = slicing.choose_slices_for_memory(net, path, tn, batch, cap,
                                                               jet.PREC_AUTO, min_count=n_sliced)
        sliced, need_fp32, _ = slicing.choose_slices_for_memory(net, path, tn, batch, cap,
                                                                jet.PREC_FP32,
                                                                min_count=len(sliced))
        n_sliced = len(sliced)
        budget = {"hbm_budget_gb": cap / 1e9, "slices_per_batch": batch,
                  "sliced_bonds": n_sliced,
                  "planned_device_gb": {"auto": need / 1e9, "fp32": need_fp32 / 1e9},
                  "rule": "fewest bonds (greedy slicer order) whose chunk plan fits the budget"}
    else:
        sliced = circuits.choose_slices(net, path, n_sliced) if n_sliced else []
    plan_s = time.perf_counter() - t0
    full_flops, log2_big = circuits.path_cost(net, path)
    forms = {}
    amps = {}
    # (name, precision, split form of AUTO's tensor-core steps)
    all_forms = (("auto", jet.PREC_AUTO, capi.PREC_FP16X3),
                 ("tuned", jet.PREC_TUNED, capi.PREC_FP16X3),
                 ("auto_tf32", jet.PREC_AUTO, capi.PREC_TF32X3),
                 ("bf16x3", jet.PREC_BF16X3, None),
                 ("fp32", jet.PREC_FP32, None))
    sliced_forms = tuple(f for f in all_forms if f[0] in args.sliced_forms.split(","))
    profiles = {}
    for name, prec, auto_form in sliced_forms:
        capi.set_auto_form(auto_form or capi.PREC_FP16X3)
        if not sliced:
            # No slices (config 0): the network is one amplitude; time the
            # reference's own flow, a TaskBasedContractor over the path, built
            # and run afresh each time (the sliced contractor would cache it).
            jet.set_precision(prec)
            info = jet.PathInfo(tn=tn, path=path)

            def run_tbc():
                tbc = jet.TaskBasedContractor(dtype="complex64")
                tbc.add_contraction_tasks(tn, info)
                tbc.add_deletion_tasks()
                tbc.contract()
                return tbc.results[0]

            for _ in range(3):
                res = run_tbc()
            reps = []
            while sum(reps) < 0.3 or len(reps) < 5:
                t1 = time.perf_counter()
                res = run_tbc()
                reps.append(time.perf_counter() - t1)
            # The same contractor contracted again and again: from the second
            # call on, Contract() replays one captured CUDA graph.
            tbc = jet.TaskBasedContractor(dtype="complex64")
            tbc.add_contraction_tasks(tn, info)
            tbc.add_deletion_tasks()
            for _ in range(3):
                tbc.contract()
            rreps = []
            while sum(rreps) < 0.3 or len(rreps) < 5:
                t1 = time.perf_counter()
                tbc.contract()
                rreps.append(time.perf_counter() - t1)
            replay_amp = complex(tbc.results[0].data[0])
            jet.set_precision(jet.PREC_FP32)
            dt = statistics.median(reps)
            dtr = statistics.median(rreps)
            flops = info.total_flops()
            forms[name] = {"slices_per_s": 1.0 / dt, "s_per_slice": dt,
                           "eff_tflops": 4.0 * flops / dt / 1e12, "slices_timed": 1,
                           "runs": len(reps), "arena_gb": 0.0,
                           "flow": "TaskBasedContractor, built and run per amplitude",
                           "replayed": {"amplitudes_per_s": 1.0 / dtr, "s_per_amplitude": dtr,
                                        "runs": len(rreps),
                                        "same_bits": replay_amp == complex(res.data[0]),
                                        "flow": "one TaskBasedContractor, contract() repeated "
                                                "(CUDA graph replay from the second call)"}}
            amps[name] = complex(res.data[0]) if hasattr(res, "data") else complex(res[0])
            slice_flops = dep_flops = flops
            continue

        def profile(sc, start, name=name):
            if args.profile_chunk and rank == 0:
                profiles[name] = sc.profile_chunk(start)

        forms[name], info = time_sliced_form(jet, tn, path, sliced, prec, batch, chunks,
                                             after=profile)
        tuned = None
        if prec == jet.PREC_TUNED:
            table = capi.autotune_table()
            tuned = {"entries": len(table)}
            for e in table:
                tuned[e["choice"]] = tuned.get(e["choice"], 0) + 1
            if args.autotune_dump and rank == 0:
                with open(args.autotune_dump, "w") as f:
                    json.dump(table, f, indent=1)
        if tuned is not None:
            forms[name]["autotune"] = tuned
        amps[name] = info["amp"]
        slice_flops = info["slice_flops"]
        dep_flops = info["slice_dependent_flops"]
    if profiles:
        with open(args.profile_chunk, "w") as f:
            json.dump(profiles, f, indent=1)

    def rel_to_fp32(f):
        if f not in amps or "fp32" not in amps:
            return None
        return abs(amps[f] - amps["fp32"]) / max(abs(amps["fp32"]), 1e-300)

    rel, rel_bf = rel_to_fp32("auto"), rel_to_fp32("bf16x3")
    # One slice in complex128 (FP64 arithmetic on the GPU) as the reference
    # for the per-slice error of both complex64 forms.
    slice_check = None
    if args.check_fp64 and sliced:
        tn128 = jet.TensorNetwork(dtype="complex128")
        for lab, sh, d in net.tensors:
            tn128.add_tensor(jet.Tensor(indices=lab, shape=sh, data=list(d), dtype="complex128"))
        sc = jet.SlicedContractorC128(tn128, path, sliced, jet.PREC_FP32)
        sc.set_batch_size(1)
        ref64 = sc.contract(0, 1)[0]
        del sc
        slice_check = {"reference": "complex128 FP64 on the GPU, slice 0",
                       "value": [ref64.real, ref64.imag]}
        for name, prec, auto_form in sliced_forms:
            capi.set_auto_form(auto_form or capi.PREC_FP16X3)
            sc = jet.SlicedContractorC64(tn, path, sliced, prec)
            sc.set_batch_size(1)
            v = sc.contract(0, 1)[0]
            slice_check["rel_err_" + name] = abs(v - ref64) / max(abs(ref64), 1e-300)
            del sc
    head = "auto" if "auto" in forms else next(iter(forms))
    line = {
        "metric": METRIC, "value": forms[head]["slices_per_s"], "unit": "slices/s",
        "n_gpus": world, "steps": 1, "warmup": 1,
        "ms_per_step": forms[head]["s_per_slice"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded circuit)",
        "config": {"workload": "config %s: %dx%d grid%s%s, %d %s, %d sliced bonds, %d slices "
                               "per batch, greedy path (2^%.1f flops, largest 2^%.1f)"
                               % (args.config, rows, cols, " minus %d site" % len(removed)
                                  if removed else "",
                                  " of qudits (d=%d, Haar unitaries)" % qd if qd != 2 else "",
                                  cycles, "layers" if qd != 2 else "cycles", n_sliced, batch,
                                  math.log2(full_flops), log2_big),
                   "slices_total": qd ** n_sliced},
        "forms": forms,
        "tc_vs_plain_speedup": (forms["auto"]["slices_per_s"] / forms["fp32"]["slices_per_s"]
                                if "auto" in forms and "fp32" in forms else None),
        "slice_flops_pathinfo": slice_flops, "slice_dependent_flops": dep_flops,
        "amplitude_sample": [amps[head].real, amps[head].imag],
        "rel_diff_auto_vs_fp32": rel,
        "rel_diff_bf16x3_vs_fp32": rel_bf,
        "rel_diff_tuned_vs_fp32": rel_to_fp32("tuned"),
        "slice_vs_fp64": slice_check,
        "plan_seconds": plan_s,
    }
    if args.bitstrings and sliced:
        line["bitstring_pass"] = run_bitstrings(args, jet, net, path, sliced, rows, cols, cycles,
                                                removed)
    if sliced:
        pi_big = circuits.path_cost(net, path, sliced)[1]
        line["slicing"] = dict(budget or {}, slices_total=qd ** n_sliced,
                               log2_largest_intermediate_per_slice=pi_big,
                               pathinfo_flops_per_slice=slice_flops)
        line["extrapolated_full_amplitude_s"] = {
            f: qd ** n_sliced / forms[f]["slices_per_s"] for f in forms}
    if rank == 0:
        print(json.dumps(line), flush=True)


def m12_leg(batch=8, chunks=4):
    """The reference's own m12 benchmark network (53 qubits, depth 12;
    examples/paper_benchmarks/data_files/m12.json, kept as a golden fixture)
    with the reference's 9-index slicing (GPU/jet_gpu_m12/jet_sliced_subset.cpp:
    53-54, 512 slices), loaded through the TensorNetworkSerializer
    counterpart and contracted by the sliced contractor in AUTO and plain
    FP32: slices/s, eff. TFLOP/s and the amplitude error of slices 0-2
    against the fixture's complex128 oracle values. Returns (record, the
    fixture's tensors and path, the sliced labels)."""
    import jet_gb300 as jet
    from jet_gb300 import capi

    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    import make_network_fixtures as mk

    ent = config_golden("m12")
    tensors, path = mk.load_network_npz(os.path.join(REPO, "tests", "golden", "m12_network.npz"))
    tnf = jet.TensorNetworkSerializer(dtype="complex64")(mk.network_json_text(tensors, path))
    sliced = ent["sliced"]
    capi.set_auto_form(capi.PREC_FP16X3)
    forms, errs = {}, {}
    for name, prec in (("auto", jet.PREC_AUTO), ("fp32", jet.PREC_FP32)):
        forms[name], info = time_sliced_form(jet, tnf.tensors, path, sliced, prec, batch, chunks)
        one = jet.SlicedContractorC64(tnf.tensors, path, sliced, prec)
        one.set_batch_size(1)
        errs[name] = {}
        for v, rec in ent["slices"].items():
            got = one.contract(int(v), 1)[0]
            want = complex(*rec["oracle_c128"])
            errs[name]["slice_" + v] = abs(got - want) / abs(want)
        del one
        forms[name]["rel_err_vs_fp64"] = max(errs[name].values())
        forms[name]["rel_err_per_slice"] = errs[name]
    out = {"workload": "m12: %d tensors, stored path of %d steps, %d sliced indices "
                       "(%d slices), %d slices per batch"
                       % (len(tensors), len(path), len(sliced), info["num_slices"], batch),
           "unit": "slices/s", "forms": forms,
           "tc_vs_plain_speedup": forms["auto"]["slices_per_s"] / forms["fp32"]["slices_per_s"],
           "slice_pathinfo_flops": info["slice_flops"],
           "extrapolated_all_slices_s": {f: info["num_slices"] / forms[f]["slices_per_s"]
                                         for f in forms},
           "error_reference": "complex128 oracle amplitudes of slices 0, 1, 2 (golden)"}
    return out, tensors, path, sliced


def run_m12(args, rank, world, local_rank):
    """m12_leg as its own bench line, with the CPU oracle (numpy complex64,
    the reference's per-step arithmetic) timed on one slice."""
    import torch

    torch.cuda.set_device(local_rank)
    batch = args.sliced_batch or 8
    rec, tensors, path, sliced = m12_leg(batch, args.sliced_chunks or 4)
    forms = rec["forms"]
    line = {"metric": METRIC, "value": forms["auto"]["slices_per_s"], "unit": "slices/s",
            "n_gpus": world, "steps": 1, "warmup": 1,
            "ms_per_step": forms["auto"]["s_per_slice"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64",
            "data": "the reference's m12 network (golden fixture of its data file)",
            "config": {"workload": rec["workload"]}}
    line.update({k: v for k, v in rec.items() if k not in ("workload", "unit")})
    if not args.no_cpu_baseline:
        from oracle import jet_oracle as jo

        tn = jo.OTensorNetwork()
        for _, lab, sh, d in tensors:
            tn.add_tensor(jo.OTensor.make(lab, sh, np.asarray(d, np.complex64), np.complex64))
        tn.slice_indices(list(sliced), 0)
        t0 = time.perf_counter()
        tn.contract(path, release=True)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "slices/s",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "slice 0 of m12 in complex64 through the numpy oracle "
                                          "(TensorNetwork::Contract restated, BLAS threads = "
                                          "host cores), %.1f s" % dt}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_m12_tbc(args, rank, world, local_rank):
    """The reference's m12 flow (GPU/jet_gpu_m12/jet_sliced_subset.cpp:
    50-101) through the TaskBasedContractor API: the m12 network sliced over
    its 9 indices, the first S slices (the reference's default: 3; here
    --sliced-batch) each added to one contractor, which shares their
    slice-independent tasks, then deletion and reduction tasks, and the
    contractor's first contract() timed (eager), then a replay of the graph
    its second call captured. The
    reduction is checked against the sum of the fixture's complex128 oracle
    amplitudes of those slices."""
    import torch

    import jet_gb300 as jet
    from jet_gb300 import capi

    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    import make_network_fixtures as mk

    torch.cuda.set_device(local_rank)
    ent = config_golden("m12")
    tensors, path = mk.load_network_npz(os.path.join(REPO, "tests", "golden", "m12_network.npz"))
    text = mk.network_json_text(tensors, path)
    n_slices = args.sliced_batch or 3
    capi.set_auto_form(capi.PREC_FP16X3)
    forms = {}
    for name, prec in (("auto", jet.PREC_AUTO), ("fp32", jet.PREC_FP32)):
        jet.set_precision(prec)
        runs, replays, shared = [], [], 0
        for rep in range(args.warmup + 3):
            tbc = jet.TaskBasedContractor(dtype="complex64")
            for v in range(n_slices):
                tnf = jet.TensorNetworkSerializer(dtype="complex64")(text)
                tnf.tensors.slice_indices(ent["sliced"], v)
                shared = max(shared, tbc.add_contraction_tasks(
                    tnf.tensors, jet.PathInfo(tnf.tensors, tnf.path.path)))
            tbc.add_deletion_tasks()
            tbc.add_reduction_task()
            t0 = time.perf_counter()
            tbc.contract()
            t1 = time.perf_counter()
            got = complex(tbc.reduction_result.data[0])
            tbc.contract()  # the second call captures the graph
            t2 = time.perf_counter()
            tbc.contract()
            t3 = time.perf_counter()
            if rep >= args.warmup:
                runs.append(t1 - t0)
                replays.append(t3 - t2)
            del tbc
        jet.set_precision(jet.PREC_FP32)
        want = [complex(*ent["slices"][str(v)]["oracle_c128"])
                for v in range(n_slices) if str(v) in ent["slices"]]
        err = (abs(got - sum(want)) / sum(abs(w) for w in want)
               if len(want) == n_slices else None)
        dt, dtr = statistics.median(runs), statistics.median(replays)
        forms[name] = {"slices_per_s": n_slices / dt, "s_per_contract": dt,
                       "replayed": {"slices_per_s": n_slices / dtr, "s_per_contract": dtr},
                       "shared_tasks": shared, "runs": len(runs),
                       "rel_err_vs_fp64": err}
    line = {"metric": METRIC, "value": forms["auto"]["slices_per_s"], "unit": "slices/s",
            "n_gpus": world, "steps": forms["auto"]["runs"], "warmup": args.warmup,
            "ms_per_step": forms["auto"]["s_per_contract"] * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c64",
            "data": "the reference's m12 network (golden fixture of its data file)",
            "config": {"workload": "m12 as jet_sliced_subset.cpp drives it: %d slices of the "
                                   "9-index slicing in one TaskBasedContractor (shared tasks, "
                                   "deletion and reduction tasks), contract() timed"
                                   % n_slices},
            "forms": forms,
            "error_reference": "sum of the complex128 oracle amplitudes of the slices (golden), "
                               "normalised by the sum of their magnitudes"}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_m10(args, rank, world, local_rank):
    """The reference's m10 benchmark network (53 qubits, depth 10;
    examples/paper_benchmarks/data_files/m10.json, kept as a golden fixture)
    contracted whole on its stored path, as GPU/jet_gpu_m10/jet_full.cpp does:
    a TaskBasedContractor built over the path, then its contract() timed, per
    amplitude, in AUTO and plain FP32; then one contractor contracted again
    and again (graph replay). Errors against the fixture's compiled-reference complex<double>
    amplitude; the CPU oracle (numpy complex64, the reference's per-step
    arithmetic) timed on the same contraction."""
    import torch

    import jet_gb300 as jet
    from jet_gb300 import capi

    sys.path.insert(0, os.path.join(REPO, "tests", "golden"))
    import make_network_fixtures as mk

    torch.cuda.set_device(local_rank)
    ent = config_golden("m10")
    tensors, path = mk.load_network_npz(os.path.join(REPO, "tests", "golden", "m10_network.npz"))
    tnf = jet.TensorNetworkSerializer(dtype="complex64")(mk.network_json_text(tensors, path))
    want = complex(*ent["ref_c128"])
    capi.set_auto_form(capi.PREC_FP16X3)
    forms = {}
    for name, prec in (("auto", jet.PREC_AUTO), ("fp32", jet.PREC_FP32)):
        jet.set_precision(prec)

        def run_tbc():
            """(contract() seconds, build seconds, amplitude): a fresh
            contractor's first, eager contract() is timed, as the reference's
            jet_full.cpp times tbc.Contract().wait() after building it."""
            t0 = time.perf_counter()
            tbc = jet.TaskBasedContractor(dtype="complex64")
            tbc.add_contraction_tasks(tnf.tensors, tnf.path)
            tbc.add_deletion_tasks()
            t1 = time.perf_counter()
            tbc.contract()
            t2 = time.perf_counter()
            return t2 - t1, t1 - t0, complex(tbc.results[0].data[0])

        for _ in range(args.warmup):
            run_tbc()
        reps, builds = [], []
        while sum(reps) < 2.0 or len(reps) < 5:
            dt, db, amp = run_tbc()
            reps.append(dt)
            builds.append(db)
        tbc = jet.TaskBasedContractor(dtype="complex64")
        tbc.add_contraction_tasks(tnf.tensors, tnf.path)
        tbc.add_deletion_tasks()
        for _ in range(args.warmup):
            tbc.contract()
        rreps = []
        while sum(rreps) < 2.0 or len(rreps) < 5:
            t1 = time.perf_counter()
            tbc.contract()
            rreps.append(time.perf_counter() - t1)
        ramp = complex(tbc.results[0].data[0])
        del tbc
        jet.set_precision(jet.PREC_FP32)
        dt, dtr = statistics.median(reps), statistics.median(rreps)
        flops = ent["pathinfo_flops"]
        forms[name] = {"amplitudes_per_s": 1.0 / dt, "s_per_amplitude": dt,
                       "eff_tflops": 4.0 * flops / dt / 1e12, "runs": len(reps),
                       "build_s": statistics.median(builds),
                       "timed": "contract() of a freshly built TaskBasedContractor (eager), "
                                "as jet_full.cpp times it; building it (build_s) untimed",
                       "rel_err_vs_fp64": abs(amp - want) / abs(want),
                       "replayed": {"amplitudes_per_s": 1.0 / dtr, "s_per_amplitude": dtr,
                                    "eff_tflops": 4.0 * flops / dtr / 1e12, "runs": len(rreps),
                                    "same_bits": ramp == amp}}
    line = {"metric": "amplitudes/s & eff. TFLOP/s of the m10 network, TC-split vs plain FP32",
            "value": forms["auto"]["amplitudes_per_s"], "unit": "amplitudes/s",
            "n_gpus": world, "steps": forms["auto"]["runs"],
            "warmup": args.warmup, "ms_per_step": forms["auto"]["s_per_amplitude"] * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64",
            "data": "the reference's m10 network (golden fixture of its data file)",
            "config": {"workload": "m10: %d tensors, stored path of %d steps, whole network "
                                   "(one amplitude) per TaskBasedContractor run"
                                   % (len(tensors), len(path))},
            "forms": forms,
            "tc_vs_plain_speedup": forms["auto"]["amplitudes_per_s"]
            / forms["fp32"]["amplitudes_per_s"],
            "pathinfo_flops": ent["pathinfo_flops"],
            "error_reference": "the compiled reference's complex<double> amplitude (golden)"}
    if not args.no_cpu_baseline:
        from oracle import jet_oracle as jo

        tn = jo.OTensorNetwork()
        for _, lab, sh, d in tensors:
            tn.add_tensor(jo.OTensor.make(lab, sh, np.asarray(d, np.complex64), np.complex64))
        t0 = time.perf_counter()
        tn.contract(path, release=True)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": "amplitudes/s",
                                "cores": os.cpu_count(), "kind": "port",
                                "sample": "the whole m10 contraction in complex64 through the "
                                          "numpy oracle (TensorNetwork::Contract restated, BLAS "
                                          "threads = host cores), %.1f s" % dt}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_grad(args, rank, world, local_rank):
    """Config 3: d Re<psi|Z_i Z_j|psi> / d(720 angles) of a 6x6, 10-layer
    RX-RZ-CZ circuit through the hand-written adjoint (light-cone-pruned
    doubled network, complex64 on the GPU, AUTO form). The value is the
    gradient rate of the evaluation captured in one CUDA graph; the eager
    forward and backward times are reported beside it, with the largest
    deviation of the graphed gradient from complex128 central finite
    differences (h = 1e-4, complex128 forward on the GPU) over seeded angles."""
    import torch

    import jet_gb300 as jet
    from jet_gb300 import autograd, circuits, expectation as ex

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    rows, cols, layers = 6, 6, 10
    rng = np.random.default_rng(SEED)
    th = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    ph = rng.uniform(0, 2 * np.pi, (layers, rows * cols))
    pair = ex.default_pair(rows, cols, SEED)
    spec = ex.zz_network(rows, cols, layers, pair)
    path = circuits.find_path(ex.numeric_network(spec, th, ph), restarts=8, seed=SEED)
    labels = [l.labels for l in spec]
    t = torch.tensor(th, dtype=torch.float32, device=dev, requires_grad=True)
    p = torch.tensor(ph, dtype=torch.float32, device=dev, requires_grad=True)
    plan = autograd.ContractionPlan(labels, [l.shape for l in spec], path)

    def step():
        t.grad = None
        p.grad = None
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        lv = ex.build_leaves(spec, t, p, dtype=torch.complex64, device=dev)
        loss = autograd.contract_network(lv, labels, path, precision=jet.PREC_AUTO, plan=plan).real
        e1.record()
        loss.backward()
        e2.record()
        torch.cuda.synchronize()
        return float(loss.item()), e0.elapsed_time(e1), e1.elapsed_time(e2)

    for _ in range(args.warmup):
        step()
    fw, bw = [], []
    for _ in range(min(args.steps, 10)):
        val, f_ms, b_ms = step()
        fw.append(f_ms)
        bw.append(b_ms)
    eager_g_t = t.grad.double().cpu().numpy()

    # The same evaluation captured once in a CUDA graph (autograd.GraphedStep)
    # and replayed: no per-step host work.
    consts = {}

    def loss_fn():
        lv = ex.build_leaves(spec, t, p, dtype=torch.complex64, device=dev, const_cache=consts)
        return autograd.contract_network(lv, labels, path, precision=jet.PREC_AUTO,
                                         plan=plan).real

    graphed = autograd.GraphedStep(loss_fn, [t, p], warmup=max(2, args.warmup))
    for _ in range(3):
        graphed.step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        graphed.step()
    e1.record()
    torch.cuda.synchronize()
    graph_ms = e0.elapsed_time(e1) / args.steps
    # The forward pass alone (no gradient bookkeeping), captured and replayed
    # the same way: the gradient is timed against it.
    fwd_graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side), torch.no_grad():
        loss_fn()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    with torch.no_grad(), torch.cuda.graph(fwd_graph):
        fwd_loss = loss_fn()
    for _ in range(3):
        fwd_graph.replay()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        fwd_graph.replay()
    e1.record()
    torch.cuda.synchronize()
    fwd_graph_ms = e0.elapsed_time(e1) / args.steps
    fwd_same = float(fwd_loss.item()) == float(graphed.loss.item())
    del fwd_graph
    g_t = graphed.grads[0].double().cpu().numpy()
    g_p = graphed.grads[1].double().cpu().numpy()
    graph_vs_eager = float(np.abs(g_t - eager_g_t).max())

    def loss64(a, b):
        lv = ex.build_leaves(spec, torch.tensor(a, device=dev), torch.tensor(b, device=dev),
                             dtype=torch.complex128, device=dev)
        return float(autograd.contract_network(lv, labels, path, precision=jet.PREC_FP32,
                                               plan=plan).real.item())

    h = 1e-4
    worst = 0.0
    picks = [(int(rng.integers(layers)), int(rng.integers(rows * cols)), w)
             for w in ("t", "p") for _ in range(6)]
    for l, q, w in picks:
        a1, b1, a2, b2 = th.copy(), ph.copy(), th.copy(), ph.copy()
        if w == "t":
            a1[l, q] += h
            a2[l, q] -= h
        else:
            b1[l, q] += h
            b2[l, q] -= h
        fd = (loss64(a1, b1) - loss64(a2, b2)) / (2 * h)
        worst = max(worst, abs(fd - (g_t if w == "t" else g_p)[l, q]))
    f_med, b_med = statistics.median(fw), statistics.median(bw)
    line = {"metric": METRIC, "value": 1e3 / graph_ms, "unit": "gradients/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": graph_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c64", "data": "synthetic (seeded angles)",
            "config": {"workload": "config 3: 6x6 grid, 10 layers RX-RZ-CZ, 720 angles, "
                                   "Re<Z_%d Z_%d>, light-cone doubled network (%d tensors)"
                                   % (pair[0], pair[1], len(spec))},
            "graph": "forward + adjoint backward captured once in a CUDA graph "
                     "(autograd.GraphedStep) and replayed",
            "forward_graph_ms": fwd_graph_ms,
            "gradient_over_forward": graph_ms / fwd_graph_ms,
            "forward_graph_same_loss": fwd_same,
            "eager": {"forward_ms": f_med, "backward_ms": b_med,
                      "backward_over_forward": b_med / f_med, "gradients_per_s":
                      1e3 / (f_med + b_med)},
            "graph_vs_eager_max_abs_diff": graph_vs_eager,
            "loss": val, "max_abs_err_vs_fd_complex128": worst, "fd_checks": len(picks)}
    if rank == 0:
        print(json.dumps(line), flush=True)


def _parse_shape(text):
    """'3^16' -> [3] * 16; '9,5,7,3' -> [9, 5, 7, 3]."""
    if "^" in text:
        d, r = text.split("^")
        return [int(d)] * int(r)
    return [int(v) for v in text.split(",")]


def run_permute(args):
    """One permute (jetgpu_permute) of a seeded random permutation (or
    --permute-perm), timed with CUDA events on the launching stream over
    --steps launches after --warmup;
    the output is compared bit for bit with torch's permute of the same
    tensor. Algorithmic traffic: one read and one write of every element."""
    import numpy as np
    import torch

    from jet_gb300 import capi

    dev = torch.device("cuda:0")
    shape = _parse_shape(args.permute_shape)
    perm = ([int(v) for v in args.permute_perm.split(",")] if args.permute_perm else
            [int(v) for v in np.random.default_rng(SEED).permutation(len(shape))])
    tdt = torch.complex128 if args.permute_dtype == "c128" else torch.complex64
    n = int(np.prod(shape))
    g = torch.Generator(device=dev)
    g.manual_seed(SEED)
    x = torch.randn(n, dtype=tdt, device=dev, generator=g)
    y = torch.empty_like(x)
    for _ in range(args.warmup):
        capi.permute(x, shape, perm, out=y)
    torch.cuda.synchronize()
    exact = bool(torch.equal(y, x.view(shape).permute(perm).contiguous().view(-1)))
    st = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with Clocks(0) as clk:
        e0.record(st)
        for _ in range(args.steps):
            capi.permute(x, shape, perm, out=y)
        e1.record(st)
        torch.cuda.synchronize()
    clocks = clk.summary()
    ms = e0.elapsed_time(e1) / args.steps
    nbytes = 2 * n * x.element_size()
    gbs = nbytes / ms / 1e6
    hbm, _, src = measured_peaks()
    print(json.dumps({
        "metric": "permute_bandwidth", "value": gbs, "unit": "GB/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "dtype": args.permute_dtype, "data": "synthetic (seeded)",
        "config": {"workload": "permute %s %s, perm %s" % (args.permute_shape, args.permute_dtype,
                                                           perm),
                   "elements": n, "l2": "input and output each larger than L2" if nbytes // 2 > 129e6
                   else "fits L2 (launch-bound case)"},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                     "frac": gbs / hbm, "peak_source": src, "traffic_algorithmic": nbytes},
        "exact": exact, "clocks": clocks}))


def run_gate(args):
    """One gate applied to a state-like tensor through jetgpu_contract (the
    skinny kernel): --gate-shape 'D^R:Q' is a tensor of R axes of dimension D
    and a gate reading Q of them (seeded positions) and writing Q new ones,
    contracted as Tensor::ContractTensors orders it (state's free axes, then
    the gate's outputs). Timed with CUDA events over --steps launches after
    --warmup; the transposing path (jetgpu_permute of the state, then
    jetgpu_multiply) is timed beside it and must give the same bits.
    Algorithmic traffic: the state read once and the output written once."""
    import numpy as np
    import torch

    from jet_gb300 import capi

    dev = torch.device("cuda:0")
    dims, q = args.gate_shape.split(":")
    shape = _parse_shape(dims)
    q = int(q)
    r, d = len(shape), shape[0]
    rng = np.random.default_rng(SEED)
    gate_axes = sorted(int(v) for v in rng.choice(r, size=q, replace=False))
    free = [i for i in range(r) if i not in gate_axes]
    a_perm = free + gate_axes
    k = n = d ** q
    m = int(np.prod([shape[i] for i in free]))
    g_shape = [d] * (2 * q)
    b_perm = list(range(q, 2 * q)) + list(range(q))  # gate labels (out..., in...)
    tdt = torch.complex128 if args.permute_dtype == "c128" else torch.complex64
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED)
    x = torch.randn(m * k, dtype=tdt, device=dev, generator=gen)
    gt = torch.randn(k * n, dtype=tdt, device=dev, generator=gen)
    y = torch.empty(m * n, dtype=tdt, device=dev)
    xt = torch.empty_like(x)
    y2 = torch.empty_like(y)
    bt = capi.permute(gt, g_shape, b_perm)
    assert capi.contract_workspace_size(shape, a_perm, g_shape, b_perm, m, n, k,
                                        capi.dtype_code(tdt), capi.PREC_FP32) == 0

    def skinny():
        capi.contract(x, shape, a_perm, gt, g_shape, b_perm, m, n, k, out=y)

    def transposing():
        capi.permute(x, shape, a_perm, out=xt)
        capi.multiply(xt, bt, m, n, k, out=y2)

    st = torch.cuda.current_stream()
    times = {}
    for name, fn in (("skinny", skinny), ("transposing", transposing)):
        for _ in range(args.warmup):
            fn()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        if name == "skinny":
            with Clocks(0) as clk:
                e0.record(st)
                for _ in range(args.steps):
                    fn()
                e1.record(st)
                torch.cuda.synchronize()
            clocks = clk.summary()
        else:
            e0.record(st)
            for _ in range(args.steps):
                fn()
            e1.record(st)
            torch.cuda.synchronize()
        times[name] = e0.elapsed_time(e1) / args.steps
    exact = bool(torch.equal(y, y2))
    nbytes = (m * k + m * n) * x.element_size()
    gbs = nbytes / times["skinny"] / 1e6
    hbm, _, src = measured_peaks()
    print(json.dumps({
        "metric": "gate_bandwidth", "value": gbs, "unit": "GB/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": times["skinny"],
        "higher_is_better": True, "dtype": args.permute_dtype, "data": "synthetic (seeded)",
        "config": {"workload": "gate on %s %s: %d-axis gate on axes %s (m %d, k %d, n %d)"
                               % (dims, args.permute_dtype, q, gate_axes, m, k, n),
                   "l2": "input and output each larger than L2" if nbytes // 2 > 129e6
                   else "fits L2 (launch-bound case)"},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                     "frac": gbs / hbm, "peak_source": src, "traffic_algorithmic": nbytes},
        "transposing_ms": times["transposing"],
        "speedup_vs_transposing": times["transposing"] / times["skinny"],
        "same_bits_as_transposing": exact, "clocks": clocks}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sliced", action="store_true",
                    help="config 1: skip the sliced legs (configs 4 and 2: AUTO vs plain FP32 "
                         "slices/s)")
    ap.add_argument("--small", action="store_true",
                    help="profiling case: rank-25 x rank-25 (M = N = 2^12, K = 2^13)")
    ap.add_argument("--kernels-only", action="store_true",
                    help="skip the plain-FP32, end-to-end and CPU legs")
    ap.add_argument("--autotune-dump", default=None,
                    help="sliced configs: write the autotuner's table (per-step candidate "
                         "times) of the tuned form to this JSON file")
    ap.add_argument("--profile-chunk", default=None,
                    help="sliced configs: write each form's per-step device times of one chunk "
                         "(SlicedContractor.profile_chunk) to this JSON file")
    ap.add_argument("--check-fp64", action="store_true",
                    help="sliced configs: also contract slice 0 in complex128")
    ap.add_argument("--form", default="auto",
                    choices=["auto", "tf32x3", "bf16x3", "fp16x3", "bf16x3_3m", "fp16x3_3m"],
                    help="split form of the config-1 step (auto: all timed, the headline is "
                         "the fastest whose error on the step is within 1e-5)")
    ap.add_argument("--sliced-forms", default="auto,tuned,auto_tf32,fp32",
                    help="forms timed by the sliced configs (comma list of auto (FP16x3 on "
                         "the tensor-core steps), auto_tf32, bf16x3, fp32)")
    ap.add_argument("--bitstrings", type=int, default=0,
                    help="sliced configs: also run the bitstring pass over this many "
                         "seeded-uniform output bitstrings (config 2: 256), timed on a sample")
    ap.add_argument("--bitstring-chunk", type=int, default=4,
                    help="bitstrings per run of the bitstring pass (alternatives of the caps)")
    ap.add_argument("--sliced-batch", type=int, default=0,
                    help="slices per batch of the sliced configs (0: the config's own)")
    ap.add_argument("--sliced-chunks", type=int, default=0,
                    help="batches timed by the sliced configs (0: the config's own)")
    ap.add_argument("--tc-chunk", type=int, default=None,
                    help="K depth accumulated in tensor memory per fold (0 = defaults)")
    ap.add_argument("--tc-persistent", type=int, default=None, choices=[0, 1],
                    help="tensor-core products: 1 one persistent CTA per SM (default), "
                         "0 one CTA per tile")
    ap.add_argument("--tc-variant", type=int, default=None,
                    help="tensor-core main loop: 0 = N 128 MMAs, 1 = N 256 MMAs")
    ap.add_argument("--config", default="1",
                    help="1 (default): the pairwise contraction; 0, 2, 4, 4q (qutrits): sliced "
                         "circuit amplitudes through the sliced executor; 3: gradients; m12: the "
                         "reference's m12 network with its own slicing; m12-tbc: m12 through the "
                         "TaskBasedContractor as the reference's driver does; m10: the reference's "
                         "m10 network contracted whole")
    ap.add_argument("--permute-shape", default=None,
                    help="time one permute instead: dims as '3^16' or '9,5,7,3' (seeded random "
                         "permutation)")
    ap.add_argument("--permute-perm", default=None,
                    help="with --permute-shape: this permutation ('2,0,1') instead of a seeded "
                         "random one")
    ap.add_argument("--permute-dtype", default="c64", choices=["c64", "c128"],
                    help="element type of --permute-shape and --gate-shape")
    ap.add_argument("--gate-shape", default=None,
                    help="time one gate applied to a state-like tensor instead: 'D^R:Q' (R axes "
                         "of dimension D, a Q-axis gate on seeded positions)")
    args = ap.parse_args()
    if args.gate_shape:
        if args.warmup < 3:
            args.warmup = 3
        run_gate(args)
        return
    if args.permute_shape:
        if args.warmup < 3:
            args.warmup = 3
        run_permute(args)
        return
    if args.warmup < 3:
        args.warmup = 3
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.config == "3":
        run_grad(args, rank, world, local_rank)
        return
    if args.config == "m12":
        run_m12(args, rank, world, local_rank)
        return
    if args.config == "m10":
        run_m10(args, rank, world, local_rank)
        return
    if args.config == "m12-tbc":
        run_m12_tbc(args, rank, world, local_rank)
        return
    if args.config != "1":
        run_sliced(args, rank, world, local_rank)
        return
    if world > 1:
        import torch

        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world, local_rank)
    if world > 1:
        import torch

        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
