"""Benchmark of the CDet integrand on GB300.

Workload: 8x8 periodic Hubbard lattice, t=1, U=4, beta=8, mu=0, subsystem A =
4x4 corner block (origin square, radius 2), Chebyshev degree 128, 65,536
seeded configurations at order n = 10 per step (uniform vertices, both spins).
One step evaluates the whole batch; `value` is configurations per second over
the whole job with the inputs resident in HBM, `e2e` the same through the
host-buffer C-ABI call with the host<->device copies inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--path both|split|fp64]
  python bench.py --impl reference ...   # the CPU integrand on the host cores

Under torchrun each rank evaluates its own 65,536 configurations (weak
scaling, no collective on the data path); timing is bracketed by a barrier and
a device synchronize and the maximum over ranks is reported.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "cdet-renyi-entanglement-hpc_gb300"))

import numpy as np  # noqa: E402

METRIC = "configs/sec at order n: batched mixed-prec vs plain FP64 on GB300 at <=1e-10 rel err"
UNIT = "configs/s"
WORKLOAD = {
    "workload": "8x8 Hubbard, 4x4 corner subsystem, Chebyshev degree 128, order n=10, "
                "65536 configurations per step (per GPU)",
    "lattice": "8x8", "U": 4, "beta": 8, "mu": 0, "mask": "origin_square r=2",
    "cheb_degree": 128, "order": 10, "batch_per_gpu": 65536,
}
BATCH = 65536
# DRAM traffic of one split_assembly launch, modelled as every coefficient
# block's slices once (a block's tiles run back to back on one SM, so its
# later tiles read them from L2) plus, per lookup, its record (u, v and
# packed slot: 24 B read) and its two Green-entry writes (8 B each, a 32-byte
# DRAM sector each: 64 B). SPLIT_TRAFFIC_RATIO is measured / model from one
# ncu capture of the small 6x6 / degree-96 case (dram__bytes_read.sum +
# dram__bytes_write.sum = 3.009 GB against a model of 3.701 GB; below 1
# because the kernel skips the zero digit slices before each K step's lead,
# profiles/split_assembly_traffic_6x6_d96_n10.md); the bench's traffic is
# that ratio times the model of its own workload.
SPLIT_TRAFFIC_RATIO = 3.009076224e9 / 3.70147328e9
SPLIT_TRAFFIC_RULE = ("model (distinct coefficient blocks x slice bytes + 88 B per lookup) x the measured/model "
                      "ratio 0.813 of the 6x6-d96 ncu capture")
ORDER = 10
L2_FLUSH_BYTES = 512 << 20
PRESET = "8x8-d128"


def workload_params():
    """The benchmark workload, or (--preset 6x6-d96) a 6x6 / half-lattice /
    degree-96 case whose 1.5 GB of tables suit profiler captures."""
    from cdet_gb300.params import CdetParams, half_lattice_mask, named_mask
    if PRESET == "6x6-d96":
        return CdetParams(n1=6, n2=6, beta="5", mu="0", u="4", alpha_up="0", alpha_down="0",
                          mask_sites=half_lattice_mask(6, 6), cheb_nu=96, cheb_nv=96)
    return CdetParams(n1=8, n2=8, beta="8", mu="0", u="4", alpha_up="0", alpha_down="0",
                      mask_sites=named_mask("origin_square", 8, 8, 2), cheb_nu=128, cheb_nv=128)


def split_model_bytes(params, lookups: int) -> float:
    """The traffic model of one split assembly launch (see SPLIT_TRAFFIC_RATIO):
    the slices of every coefficient block the lookups reach (twisted: 4 S^2
    site pairs, ordinary: its replica-(0,0) S^2, two branches each; all of
    them at the benchmark batch) plus 88 B per lookup."""
    s2 = params.sites ** 2
    ksteps = (params.cheb_nv + 15) // 16
    row_chunks = (params.cheb_nu + 127) // 128
    blocks = (4 * s2 + s2) * 2
    return blocks * row_chunks * ksteps * 32768.0 + 88.0 * lookups


def split_dram_bytes(params, lookups: int):
    return None if SPLIT_TRAFFIC_RATIO is None else SPLIT_TRAFFIC_RATIO * split_model_bytes(params, lookups)


def line_config(head: str, world: int) -> dict:
    """The `config` of the bench line, shared by both arms so that the
    reference arm's line names the same workload (the profiling preset and a
    non-default batch name themselves)."""
    if PRESET == "6x6-d96":
        work = {"workload": f"6x6 Hubbard U=4 beta=5, half-lattice subsystem, Chebyshev degree 96, order n=10, "
                            f"{BATCH} configurations per step (per GPU): the profiling preset, not the benchmark",
                "lattice": "6x6", "U": 4, "beta": 5, "mu": 0, "mask": "half lattice", "cheb_degree": 96,
                "order": ORDER, "batch_per_gpu": BATCH}
        return dict(work, path=head, parallelism=f"replicas x{world}", l2="flushed between steps (512 MiB write)")
    work = dict(WORKLOAD)
    if BATCH != WORKLOAD["batch_per_gpu"]:
        work["workload"] = work["workload"].replace("65536", str(BATCH))
        work["batch_per_gpu"] = BATCH
    return dict(work, path=head, parallelism=f"replicas x{world}",
                l2="flushed between steps (512 MiB write); tables 8.6 GB > L2")


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), p.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during a timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.device_index = device_index
        self.proc = None
        self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device_index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.out.flush()
        self.out.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.out.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, flag in zip(names, f[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        os.unlink(self.out.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def time_cpu_integrand(params, tables, vertices, orders, threads):
    """The C restatement of the reference integrand (oracle/) on the host
    cores: returns (seconds, values)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from bindings import Oracle
    orc = Oracle(params.runtime_scalars(), tables)
    t0 = time.perf_counter()
    values, _ = orc.integrand_batch(vertices, orders, threads=threads)
    return time.perf_counter() - t0, values


def derived_rates(configs_per_s: float, order: int) -> dict:
    """The integrand rate in the counting conventions of the workload
    description: principal-minor subsets (2^n per matrix, 4 matrices per
    configuration: 2 table sets x up/down, counted even where up and down
    share one table) and subset pairs (3^n per recursion, 2 recursions per
    configuration)."""
    return {"principal_minor_subsets_per_s": configs_per_s * 4 * 2 ** order,
            "subset_pairs_per_s": configs_per_s * 2 * 3 ** order,
            "conventions": "4 x 2^n principal-minor subsets and 2 x 3^n subset pairs per configuration"}


def precision_by_order(params, tables, host, integrand, device, threads, per_order):
    """The split and FP64 forms at every order 1..10 of the workload (seeded
    configurations of the same lattice, tables and vertex distribution),
    against the oracle's long double truth (the checker, not a measured path),
    with the round-off filter on (the reference's default) and off, in the
    three error forms of oracle/precision.py; and the double-double form
    (INTEGRAND_REAL=double_double, the reference's own high-precision mode)
    with its default filter. The contract the line states: condition-scaled
    error <= 1e-10 at every order."""
    import torch
    from cdet_gb300.integrand import CdetIntegrand
    from cdet_gb300.synthetic import uniform_configurations
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from bindings import Oracle
    from precision import error_forms
    orc = Oracle(params.runtime_scalars(), host)
    contexts = {"filter_on": integrand,
                "filter_off": CdetIntegrand(dataclasses.replace(params, z_safety="0"), tables, device=device)}
    dev = torch.device("cuda", device)
    out = {"configs_per_order": per_order,
           "contract": "condition_scaled <= 1e-10: |x - truth| / (M_twisted + 2 M_ordinary), M = prefactor x the "
                       "connected recursion on absolute values (the magnitude of every term of the value); the "
                       "relative error is ill-posed at high order (the sum cancels by factors up to 1e19 at order "
                       "10), and with the filter on (the reference default) the FP64 value itself is far off at "
                       "order 10 (fp64_vs_truth_filter_on)",
           "truth": "oracle long double integrand without the round-off filter, pinned to the reference's "
                    "VECTOR_REAL=long_double / INTEGRAND_REAL=double_double mode",
           "orders": {}}
    worst = 0.0
    t0 = time.perf_counter()
    for n in range(1, ORDER + 1):
        v = uniform_configurations(31000 + n, per_order, n)
        o = np.full(per_order, n, np.int32)
        truth, parts, st = orc.integrand_ld_parts_batch(v, o, threads=threads)
        dv, do = torch.from_numpy(v).to(dev), torch.from_numpy(o).to(dev)
        vals = torch.empty(per_order, dtype=torch.float64, device=dev)
        status = torch.empty(per_order, dtype=torch.int32, device=dev)
        got = {}
        for filt, ctx in contexts.items():
            for path in ("split", "fp64"):
                ctx.set_assembly(path)
                ctx.integrand_device(dv, do, vals, status)
                torch.cuda.synchronize(dev)
                got[(filt, path)] = (vals.cpu().numpy().copy(), status.cpu().numpy().copy())
        integrand.set_integrand_real("double_double")
        integrand.set_integrand_form("staged")  # the lane layout, as the timed batch runs it
        for path, key in (("fp64", "dd"), ("split", "dd_split")):  # the reference's mode; on split Green matrices
            integrand.set_assembly(path)
            integrand.integrand_device(dv, do, vals, status)
            torch.cuda.synchronize(dev)
            got[("filter_on", key)] = (vals.cpu().numpy().copy(), status.cpu().numpy().copy())
        integrand.set_integrand_real("double")
        integrand.set_integrand_form("auto")
        ok = st == 0
        for key in got:
            ok &= got[key][1] == 0
        entry = {}
        for filt in contexts:
            for path in ("split", "fp64"):
                entry[f"{path}_vs_truth_{filt}"] = error_forms(got[(filt, path)][0], truth, parts, ok)
                worst = max(worst, entry[f"{path}_vs_truth_{filt}"]["condition_scaled"]["max"])
        entry["dd_vs_truth_filter_on"] = error_forms(got[("filter_on", "dd")][0], truth, parts, ok)
        entry["dd_split_vs_truth_filter_on"] = error_forms(got[("filter_on", "dd_split")][0], truth, parts, ok)
        entry["split_vs_fp64_filter_on"] = error_forms(got[("filter_on", "split")][0],
                                                       got[("filter_on", "fp64")][0], parts, ok)
        entry["configs"] = int(ok.sum())
        out["orders"][str(n)] = entry
    integrand.set_assembly("split")
    contexts["filter_off"].close()
    out["worst_condition_scaled"] = worst
    out["contract_met"] = bool(worst <= 1e-10)
    out["seconds"] = time.perf_counter() - t0
    return out


def time_dd_forms(integrand, d_vertices, d_orders, stream, args, flush):
    """The double-double integrand (the reference's INTEGRAND_REAL=double_double
    mode) on the same batches: with the FP64 assembly (the reference's mode, bit
    for bit; its Clenshaw sums make a step long, so 8,192 configurations of the
    batch) and on the split assembly's Green matrices (the whole batch); CUDA
    events around `steps` evaluations after one warm-up each."""
    import torch
    out = {}
    for assembly, count in (("split", BATCH), ("fp64", min(BATCH, 8192))):
        integrand.set_assembly(assembly)
        integrand.set_integrand_real("double_double")
        v = [d_vertices[k][:count].contiguous() for k in range(args.steps)]
        o = d_orders[:count].contiguous()
        vals = torch.empty(count, dtype=torch.float64, device=o.device)
        st = torch.empty(count, dtype=torch.int32, device=o.device)
        integrand.integrand_device(v[0], o, vals, st, stream)
        torch.cuda.synchronize(o.device)
        integrand.profile(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for k in range(args.steps):
            flush.zero_()
            integrand.integrand_device(v[k], o, vals, st, stream)
        e1.record(stream)
        torch.cuda.synchronize(o.device)
        stage_ms, _ = integrand.profile_read()
        integrand.profile(False)
        integrand.set_integrand_real("double")
        ms = e0.elapsed_time(e1) / args.steps
        out[f"{assembly}_assembly"] = {
            "value": count / (ms / 1e3), "unit": UNIT, "configs_per_step": count, "ms_per_step": ms,
            "stages_ms_per_step": {"assembly": (stage_ms[0] + stage_ms[1]) / args.steps,
                                   "minors_and_cdet_dd": (stage_ms[2] + stage_ms[3]) / args.steps},
            "flagged_configs": int((st.cpu().numpy() & 5).astype(bool).sum())}
    integrand.set_assembly("split")
    out["note"] = ("fp64_assembly is the reference's INTEGRAND_REAL=double_double mode with VECTOR_REAL=double, "
                   "bit-identical to it; split_assembly runs the same double-double recursion on the tensor-core "
                   "Green matrices; their errors per order are in precision_by_order (dd_vs_truth_filter_on "
                   "is the reference mode's)")
    return out


def run_reference(args):
    """--impl reference: the CPU integrand timed on the host cores."""
    from cdet_gb300 import replicas
    if replicas.rank_info()[1] != 0:
        return  # under torchrun, rank 0 alone times the host cores
    import torch
    from cdet_gb300.synthetic import uniform_configurations
    from cdet_gb300.tables import build_tables
    params = workload_params()
    device = "cuda" if torch.cuda.is_available() else "cpu"
    tables = build_tables(params, device=device)
    host = {k: {kk: vv.cpu().numpy() for kk, vv in t.items()} for k, t in tables.items()}
    if tables["twisted_down"] is tables["twisted_up"]:
        host["twisted_down"] = host["twisted_up"]
        host["ordinary_down"] = host["ordinary_up"]
    del tables
    threads = cpu_threads()
    sample = args.cpu_sample or 64 * threads
    for w in range(args.warmup):
        v = uniform_configurations(700 + w, max(threads, 16), ORDER)
        time_cpu_integrand(params, host, v, np.full(v.shape[0], ORDER, np.int32), threads)
    total = 0.0
    for k in range(args.steps):
        v = uniform_configurations(9000 + k, sample, ORDER)
        dt, _ = time_cpu_integrand(params, host, v, np.full(sample, ORDER, np.int32), threads)
        total += dt
    value = args.steps * sample / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded uniform vertices)",
        # the workload's config, with the sample this arm times per step of it
        "config": dict(line_config("split", args.gpus), reference_batch_per_step=sample),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "batch_per_step": sample,
                         "sample": f"{sample} configurations per step of the workload's 65,536 "
                                   f"(same lattice, tables, order and vertex distribution), "
                                   f"{threads} threads (C restatement of the reference integrand, "
                                   "bit-identical to it on the golden vectors)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_gpu(args):
    import torch
    import torch.distributed as dist
    from cdet_gb300.integrand import CdetIntegrand
    from cdet_gb300.synthetic import uniform_configurations
    from cdet_gb300.tables import build_tables

    from cdet_gb300 import replicas
    world, rank, local_rank = replicas.rank_info()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)

    params = workload_params()
    tables = build_tables(params, device=str(dev))
    integrand = CdetIntegrand(params, tables, device=local_rank)
    integrand.reserve(BATCH, ORDER)
    paths = ["fp64", "split"] if args.path == "both" else [args.path]
    if "split" in paths:
        integrand.set_assembly("split")
        integrand.prepare_split()  # slice the tables outside any timed region

    # K + W distinct batches, resident in HBM before timing; each rank its own seeds
    n_batches = args.steps + args.warmup
    host_batches = [uniform_configurations(replicas.batch_seed(rank, s), BATCH, ORDER) for s in range(n_batches)]
    d_vertices = [torch.from_numpy(v).to(dev) for v in host_batches]
    d_orders = torch.full((BATCH,), ORDER, dtype=torch.int32, device=dev)
    d_values = torch.empty(BATCH, dtype=torch.float64, device=dev)
    d_status = torch.empty(BATCH, dtype=torch.int32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    def max_over_ranks(x: float) -> float:
        return replicas.max_over_ranks(x, world, dev)

    # the clock sampler starts before the warm-up so that nvidia-smi's start-up
    # is over when the timed regions begin
    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(2.0)

    def timed(path):
        """W untimed steps, then K timed steps (CUDA events on the launching
        stream, barrier + synchronize on both sides); returns the elapsed ms
        (max over ranks), per-stage kernel ms, launches, last values/status."""
        integrand.set_assembly(path)
        integrand.set_integrand_form(args.integrand_form)
        for w in range(args.warmup):
            flush.zero_()
            integrand.integrand_device(d_vertices[args.steps + w], d_orders, d_values, d_status, stream)
        barrier()
        integrand.profile(True)
        barrier()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record(stream)
        for k in range(args.steps):
            flush.zero_()  # L2 flush between steps
            integrand.integrand_device(d_vertices[k], d_orders, d_values, d_status, stream)
        stop.record(stream)
        barrier()
        elapsed = max_over_ranks(start.elapsed_time(stop))
        stage_ms, launches = integrand.profile_read()
        integrand.profile(False)
        tuned_forms[path] = (integrand.integrand_form_tuned(ORDER, BATCH) if args.integrand_form == "auto"
                             else {"form": args.integrand_form, "chosen_by": "--integrand-form"})
        return elapsed, stage_ms, launches, d_values.cpu().numpy(), d_status.cpu().numpy()

    tuned_forms = {}
    results = {path: timed(path) for path in paths}
    clock_info = clocks.stop()
    # tcgen05.mma instructions and slice bytes of the last split assembly (one launch)
    split_counters = integrand.split_counters() if "split" in paths else (0, 0)
    head = "split" if "split" in paths else "fp64"
    elapsed_ms, stage_ms, launches, values, status = results[head]

    # end to end through the host-buffer C-ABI call, pinned host buffers
    integrand.set_assembly(head)
    pinned_v = [torch.from_numpy(v).pin_memory() for v in host_batches[:args.steps]]
    pinned_o = torch.full((BATCH,), ORDER, dtype=torch.int32).pin_memory()
    pinned_out = torch.empty(BATCH, dtype=torch.float64).pin_memory()
    pinned_st = torch.empty(BATCH, dtype=torch.int32).pin_memory()
    lib = integrand._lib
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        rc = lib.cdet_integrand_host(integrand._ctx, pinned_v[k].data_ptr(), pinned_o.data_ptr(),
                                     BATCH, ORDER, pinned_out.data_ptr(), pinned_st.data_ptr())
        if rc not in (0, 4):
            raise RuntimeError("host-buffer evaluation failed: " + lib.cdet_last_error().decode())
    barrier()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    # both loops end on batch steps-1: the host-buffer values must equal the device ones
    e2e_match = bool(np.array_equal(pinned_out.numpy().view(np.uint64), values.view(np.uint64)))

    total_configs = BATCH * args.steps * world
    value = replicas.job_throughput(BATCH, args.steps, world, elapsed_ms / 1e3)
    e2e_value = replicas.job_throughput(BATCH, args.steps, world, e2e_s)
    hbm_peak, bf16_peak, peak_kind = peaks()
    nu, nv = params.cheb_nu, params.cheb_nv
    lookups = BATCH * 2 * ORDER * ORDER  # table sets x entries (up and down share one table)

    def per_step(ms, path):
        # the queue form runs minors and CDet in one kernel: one stage
        stages = {"split_prep": ms[0] / args.steps, "assembly": ms[1] / args.steps}
        if tuned_forms.get(path, {}).get("form") == "queue":
            stages["minors_and_cdet"] = (ms[2] + ms[3]) / args.steps
        else:
            stages.update({"minors": ms[2] / args.steps, "cdet": ms[3] / args.steps})
        return stages

    if head == "split":
        # algorithmic work of the assembly (2 nu nv flops per lookup: the
        # bilinear Chebyshev sum; 2 sets x n^2 lookups per configuration, one
        # table per set since up and down share it) against the dense tensor
        # peak; the emulation's own tensor work (the MMAs the kernel issued,
        # counted on the device) is reported beside it
        per_launch_ms = stage_ms[1] / args.steps
        flops = lookups * 2.0 * nu * nv
        achieved = flops / (per_launch_ms / 1e3) / 1e12
        mma_columns, streamed = split_counters
        issued_tflops = mma_columns * 2.0 * 128 * 16 / (per_launch_ms / 1e3) / 1e12
        roofline = {"kernel": "split_assembly (tcgen05 fp16 digit slices)", "bound": "tensor",
                    "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                    "frac": achieved / bf16_peak,
                    "peak_source": f"{peak_kind} (MEASURED_PEAKS.json bf16_tflops, burst; fp16 dense rate is the same)",
                    "algorithmic": "lookups x 2 x nu x nv (2 sets x n^2 lookups per configuration)",
                    "traffic": split_dram_bytes(params, lookups),
                    "traffic_model_bytes": split_model_bytes(params, lookups),
                    "traffic_rule": SPLIT_TRAFFIC_RULE,
                    "tcgen05_mma_columns_per_launch": mma_columns,
                    "tensor_issue_tflops": issued_tflops,
                    "tensor_issue_frac": issued_tflops / bf16_peak,
                    "tensor_issue_note": "accumulator columns written by the M=128 K=16 fp16 MMAs the kernel "
                                         "issued (counted on the device), 2*128*16 flops each: the emulation's "
                                         "tensor work, not the algorithm's",
                    "slice_bytes_streamed_per_launch": streamed}
    else:
        per_launch_ms = stage_ms[1] / args.steps
        alg_bytes = lookups * 8 * nu * nv
        achieved = alg_bytes / (per_launch_ms / 1e3) / 1e9
        roofline = {"kernel": "green_assembly_fp64", "bound": "hbm", "achieved": achieved,
                    "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                    "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)", "traffic": None,
                    "fp64_pipe_frac": lookups * 3.0 * nu * nv / (per_launch_ms / 1e3) / 504e9}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64 (split fp16-digit tcgen05 assembly, FP64 minors and CDet)" if head == "split" else "f64",
        "data": "synthetic (seeded uniform vertices, tables from the in-tree precompute)",
        "config": line_config(head, world),
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": BATCH * ORDER * 4 * 8 + BATCH * 4,
                "d2h_bytes_per_step": BATCH * 8 + BATCH * 4},
        "gpu_launches": int(launches),
        "stages_ms_per_step": per_step(stage_ms, head),
        "integrand_form": tuned_forms.get(head),
        "roofline": roofline,
        "clocks": clock_info,
        "derived": derived_rates(value, ORDER),
        "flagged_configs": int((status & 5).astype(bool).sum()),
        "fpm_fallbacks": int((status & 2).astype(bool).sum()),
        "e2e_bit_identical": e2e_match,
    }
    if "fp64" in results:
        f_ms, f_stage, _, f_values, _ = results["fp64"]
        line["fp64_path"] = {"value": total_configs / (f_ms / 1e3), "unit": UNIT,
                             "ms_per_step": f_ms / args.steps, "stages_ms_per_step": per_step(f_stage, "fp64"),
                             "integrand_form": tuned_forms.get("fp64"),
                             "bit_identical_to_reference": None}
        if head == "split":
            line["split_over_fp64"] = value / line["fp64_path"]["value"]
            ok = f_values != 0
            rel = np.abs(values[ok] - f_values[ok]) / np.abs(f_values[ok])
            line["split_vs_fp64_rel_err_order10"] = {
                "median": float(np.median(rel)), "p90": float(np.percentile(rel, 90)),
                "note": "FP64 round-off floor at order 10 (any 1-ulp change of the Green entries "
                        "moves the FP64 integrand by this much); see precision_by_order"}
    if rank == 0 and head == "split":
        # Green-matrix agreement of the two assemblies on a 2048-configuration sample
        sample = d_vertices[0][:2048].contiguous()
        so = d_orders[:2048].contiguous()
        integrand.set_assembly("fp64")
        g64, _, _ = integrand.assemble(sample, so)
        integrand.set_assembly("split")
        gsp, _, _ = integrand.assemble(sample, so)
        torch.cuda.synchronize(dev)
        scale = g64.abs().amax(dim=3, keepdim=True).clamp_min(1e-300)
        line["green_split_vs_fp64_max_rel"] = float(((gsp - g64).abs() / scale).max().item())
    if rank == 0 and head == "split" and not args.no_dd:
        line["dd_path"] = time_dd_forms(integrand, d_vertices, d_orders, stream, args, flush)

    if rank == 0 and not args.no_cpu_baseline:
        host = {k: {kk: vv.cpu().numpy() for kk, vv in t.items()} for k, t in tables.items()}
        if tables["twisted_down"] is tables["twisted_up"]:
            host["twisted_down"] = host["twisted_up"]
        if tables["ordinary_down"] is tables["ordinary_up"]:
            host["ordinary_down"] = host["ordinary_up"]
        threads = cpu_threads()
        sample = args.cpu_sample or 64 * threads
        v = host_batches[0][:sample]
        dt, cpu_values = time_cpu_integrand(params, host, v, np.full(sample, ORDER, np.int32), threads)
        integrand.set_assembly("fp64")
        integrand.integrand_device(d_vertices[0], d_orders, d_values, d_status, stream)
        torch.cuda.synchronize(dev)
        gpu_first = d_values.cpu().numpy()[:sample]
        line["cpu_baseline"] = {
            "value": sample / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {sample} configurations of the first timed batch, {threads} threads, "
                      f"{dt:.1f} s wall (C restatement of the reference integrand)",
            "bit_identical_to_gpu_fp64_path": bool(np.array_equal(cpu_values.view(np.uint64),
                                                                  gpu_first.view(np.uint64))),
        }
        if "fp64_path" in line:
            # the oracle equals the reference bit for bit on every golden vector
            line["fp64_path"]["bit_identical_to_reference"] = line["cpu_baseline"]["bit_identical_to_gpu_fp64_path"]
            line["fp64_path"]["bit_identical_checked_on"] = (f"{sample} configurations of the first timed batch "
                                                             "against the oracle")
        if head == "split" and not args.no_precision:
            line["precision_by_order"] = precision_by_order(params, tables, host, integrand, local_rank, threads,
                                                            args.precision_configs)
    if rank == 0 and "dd_path" in line and "fp64_path" in line:
        # the literal contract: relative error <= 1e-10 at every order, met by
        # the double-double recursion on the split assembly's Green matrices
        dd = line["dd_path"]["split_assembly"]
        summary = {"form": "split tcgen05 assembly + double-double minors and CDet recursion (lighter "
                           "double-double steps: FMA products, one renormalisation per sum; lane layout)",
                   "value": dd["value"], "unit": UNIT, "ms_per_step": dd["ms_per_step"],
                   "over_fp64_path": dd["value"] / line["fp64_path"]["value"]}
        if "precision_by_order" in line:
            orders = line["precision_by_order"]["orders"]
            rel = [orders[str(n)]["dd_split_vs_truth_filter_on"]["relative"]["max"] for n in range(2, ORDER + 1)]
            summary["worst_relative_error_orders_2_10"] = max(rel)
            summary["worst_combine_scaled_error_order_1"] = \
                orders["1"]["dd_split_vs_truth_filter_on"]["combine_scaled"]["max"]
            summary["contract_met"] = bool(max(rel) <= 1e-10 and summary["worst_combine_scaled_error_order_1"] <= 1e-10)
            summary["against"] = "the oracle's long double truth, pinned to the reference's high-precision mode"
        line["at_1e-10_relative"] = summary
    if rank == 0:
        print(json.dumps(line))
    integrand.close()
    if world > 1:
        dist.destroy_process_group()


def run_mcmcmc(args):
    """--mcmcmc: the device-resident MCMCMC run (a separate line, not the
    headline): 6x6 / U=2 / beta=6 / half lattice / degree 96, orders 1..8
    (envelope 9), --chains chains (128 by default) on a factorized histogram
    seed learned on the GPU, lambda adaptation during warmup, then timed
    production steps (each updating every chain's long-double statistics), for
    both assemblies; the oracle's single-threaded histogram chain beside it."""
    import torch
    from cdet_gb300.integrand import CdetIntegrand
    from cdet_gb300.mcmcmc import STREAM_TAG, McmcmcChains, jackknife_ratios, learn_histogram
    from cdet_gb300.params import CdetParams, half_lattice_mask
    from cdet_gb300.synthetic import derive_seed
    from cdet_gb300.tables import build_tables
    params = CdetParams(n1=6, n2=6, beta="6", mu="0", u="2", alpha_up="0", alpha_down="0",
                        mask_sites=half_lattice_mask(6, 6), cheb_nu=96, cheb_nv=96)
    env, omin, omax = 9, 1, 8
    lambdas = [0.0] + [1.0] * 8 + [0.0]
    chains_n = args.chains
    steps = args.mcmcmc_steps
    warmup = max(args.warmup, 100)
    hist = dict(learning_steps=64, tau_bins=16, uniform_mix=0.05, pseudo_count=0.0)
    tables = build_tables(params, device="cuda")
    gpu = CdetIntegrand(params, tables)
    out = {"metric": "MCMCMC chain-steps/s (histogram seed, envelope 9, orders 1..8)", "unit": "chain-steps/s",
           "higher_is_better": True, "n_gpus": 1, "steps": steps, "warmup": warmup,
           "config": {"workload": "6x6 Hubbard U=2 beta=6 half lattice, degree 96, envelope 9, orders 1..8, "
                                  "factorized histogram seed, lambda adaptation every 50 warmup steps",
                      "chains": chains_n, "histogram": hist},
           "data": "synthetic (seeded chains, tables from the in-tree precompute)"}
    for path in ("fp64", "split"):
        gpu.set_assembly(path)
        t0 = time.perf_counter()
        tau, space, rep, _ = learn_histogram(gpu, omin, omax, env, hist["learning_steps"], hist["tau_bins"],
                                             hist["uniform_mix"], hist["pseudo_count"], 20261203)
        learn_s = time.perf_counter() - t0
        seeds = [derive_seed(20261203, STREAM_TAG, i) for i in range(chains_n)]
        chains = McmcmcChains(gpu, omin, omax, env, seeds, lambdas, adapt_interval=50)
        chains.set_histogram(hist["tau_bins"], tau, space, rep)
        chains.run(warmup, warmup=True)
        chains.end_warmup()
        torch.cuda.synchronize()
        l0, g0 = chains.launch_count()
        t0 = time.perf_counter()
        chains.run(steps, warmup=False)
        dt = time.perf_counter() - t0
        l1, g1 = chains.launch_count()
        jack = jackknife_ratios(chains.results(), omin, omax, 1)
        # the same chains continued with every Green pair evaluated each step
        # (the values do not change), then the fraction of pairs reused
        chains.set_green_reuse(False)
        n_off = max(20, steps // 4)
        chains.run(5, warmup=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        chains.run(n_off, warmup=False)
        dt_off = time.perf_counter() - t0
        chains.set_green_reuse(True)
        rec = chains.run(50, warmup=False, record=True)
        kept = np.vectorize(lambda m: bin(int(m)).count("1"))(rec["chosen"]).astype(np.float64)
        out[path] = {"ratios_to_order1": [float(x) for x in jack["ratio"][omin:omax + 1]],
                     "jackknife_errors": [float(x) for x in jack["error"][omin:omax + 1]],
                     "value": chains_n * steps / dt, "ms_per_step": 1e3 * dt / steps,
                     "hours_for_1e5_steps": dt / steps * 1e5 / 3600, "histogram_learning_s": learn_s,
                     "gpu_launches": l1 - l0, "graph_steps": g1 - g0,
                     "green_reuse": {"ms_per_step_without": 1e3 * dt_off / n_off,
                                     "pairs_reused_fraction": float((kept ** 2).mean() / env ** 2),
                                     "note": "production steps copy the Green entries of pairs of retained "
                                             "vertices from the previous step; without: every pair evaluated"}}
        chains.close()
    out["value"] = out["split"]["value"]
    out["gpu_launches"] = out["split"]["gpu_launches"]
    # split-assembly chains against FP64-assembly chains (the reference's
    # chains): per order, the difference of the ratios to order 1 in units
    # of the combined chain-level jackknife error
    dz = []
    for k in range(omax - omin + 1):
        a, b = out["split"], out["fp64"]
        sigma = float(np.hypot(a["jackknife_errors"][k], b["jackknife_errors"][k]))
        dz.append((a["ratios_to_order1"][k] - b["ratios_to_order1"][k]) / sigma if sigma > 0 else None)
    out["split_vs_fp64_ratio_delta_over_sigma"] = dz
    if not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        from bindings import Oracle
        host = {k: {kk: vv.cpu().numpy() for kk, vv in t.items()} for k, t in tables.items()}
        orc = Oracle(params.runtime_scalars(), host)
        tau, space, rep, _ = orc.learn_histogram(omin, omax, env, 4, hist["tau_bins"], hist["uniform_mix"],
                                                 hist["pseudo_count"], 20261203)
        t0 = time.perf_counter()
        n = 6
        orc.mcmcmc_chain(omin, omax, env, lambdas, 0, 1000, 0.25, n, derive_seed(20261203, STREAM_TAG, 0),
                         histogram=(hist["tau_bins"], tau, space, rep))
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / dt, "unit": "chain-steps/s", "cores": 1, "kind": "port",
                               "sample": f"one histogram-seeded chain, {n} production steps (C restatement of "
                                         "the reference chain)"}
    print(json.dumps(out))


def run_mixed(args):
    """--mixed: a batch of uneven orders (a separate line, not the headline):
    6x6 / U=4 / beta=5 / half lattice / degree 96, 64 chains x 256 proposals
    = 16,384 configurations per step with orders 1..10 drawn from a truncated
    geometric distribution (p = 0.3), through the device entry point with the
    inputs resident; FP64 (bit-identical) and split forms. Each form is timed
    staged (minors kernel, a[] in HBM, CDet kernel), as the persistent queue
    kernel (one and two warps per configuration) and under the autotuner,
    whose kept choice gives the line's value; all forms' values are checked
    bit for bit against the staged form's."""
    import torch
    from cdet_gb300.integrand import CdetIntegrand
    from cdet_gb300.params import CdetParams, half_lattice_mask
    from cdet_gb300.synthetic import truncated_geometric_orders, uniform_configurations
    from cdet_gb300.tables import build_tables
    params = CdetParams(n1=6, n2=6, beta="5", mu="0", u="4", alpha_up="0", alpha_down="0",
                        mask_sites=half_lattice_mask(6, 6), cheb_nu=96, cheb_nv=96)
    batch, nmax = 64 * 256, 10
    gpu = CdetIntegrand(params, build_tables(params, device="cuda"))
    v = torch.from_numpy(uniform_configurations(20261203, batch, nmax)).cuda()
    o = torch.from_numpy(truncated_geometric_orders(20261204, batch, 0.3, nmax)).cuda()
    vals = torch.empty(batch, dtype=torch.float64, device="cuda")
    st = torch.empty(batch, dtype=torch.int32, device="cuda")
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.int32, device="cuda")  # 512 MiB > L2
    out = {"metric": "configs/s, mixed orders 1..10 (truncated geometric p=0.3)", "unit": "configs/s",
           "higher_is_better": True, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "config": {"workload": "6x6 Hubbard U=4 beta=5 half lattice, degree 96, 64 chains x 256 proposals "
                                  "= 16,384 configurations per step, orders 1..10 truncated geometric p=0.3",
                      "order_histogram": np.bincount(o.cpu().numpy(), minlength=nmax + 1)[1:].tolist(),
                      "l2": "flushed between steps (512 MiB write)"},
           "data": "synthetic (seeded uniform vertices, tables from the in-tree precompute)"}
    values = {}
    forms = (("staged", {}), ("queue", {}), ("queue", {"pair": True}), ("auto", {}))
    for path in ("fp64", "split"):
        gpu.set_assembly(path)
        per_form = []
        for form, shape in forms:
            gpu.set_integrand_form(form, **shape)
            for _ in range(args.warmup):  # under "auto" the first call measures the candidates
                gpu.integrand_device(v, o, vals, st)
            torch.cuda.synchronize()
            total = 0.0
            for _ in range(args.steps):
                flush.fill_(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                gpu.integrand_device(v, o, vals, st)
                e1.record()
                torch.cuda.synchronize()
                total += e0.elapsed_time(e1)
            got = vals.cpu().numpy().copy()
            if path not in values:
                values[path] = got
            entry = {"form": form, **shape, "ms_per_step": total / args.steps,
                     "configs_per_s": batch * args.steps / (total / 1e3),
                     "gpu_launches": gpu.last_launch_count(),
                     "bit_identical_to_staged": bool(np.array_equal(got.view(np.uint64),
                                                                    values[path].view(np.uint64)))}
            if form == "auto":
                entry["tuned"] = gpu.integrand_form_tuned(nmax, batch)
            per_form.append(entry)
        auto = per_form[-1]
        out[path] = {"value": auto["configs_per_s"], "ms_per_step": auto["ms_per_step"],
                     "gpu_launches": auto["gpu_launches"], "tuned": auto["tuned"], "forms": per_form}
    out["value"] = out["split"]["value"]
    # per order: relative error of each configuration, and the normwise error
    # max |split - fp64| / max |fp64| over the configurations of that order
    orders = o.cpu().numpy()
    per_order = {}
    for n in range(1, nmax + 1):
        sel = orders == n
        f, sp = values["fp64"][sel], values["split"][sel]
        rel = np.abs(sp - f) / np.maximum(np.abs(f), 1e-300)
        per_order[str(n)] = {"configs": int(sel.sum()), "median_rel": float(np.median(rel)),
                             "p90_rel": float(np.percentile(rel, 90)),
                             "normwise": float(np.abs(sp - f).max() / max(np.abs(f).max(), 1e-300)),
                             "max_abs_fp64": float(np.abs(f).max()),
                             "max_abs_diff": float(np.abs(sp - f).max())}
    out["split_vs_fp64_err_by_order"] = per_order
    out["note"] = ("order 1: twisted - 2 ordinary cancels, so its values are round-off residue of the "
                   "diagonal terms (compare max_abs_diff with the other orders' magnitudes)")
    print(json.dumps(out))


def run_stress(args):
    """--stress: the high-order stress case (a separate line, not the
    headline): 12x12 lattice, t=1, U=6, beta=10, mu=-0.5, subsystem A = the
    6x12 half lattice, Chebyshev degree 192, 8,192 configurations at order 14
    per step. Degree 192 runs the split assembly as 2 x 2 sub-blocks of each
    coefficient block. The tables (98 GB in the reference layout) and their
    split slices (163 GB) are resident together; the FP64 and split forms
    are timed on the same batches. With --stress-small the same kernels run
    on a 3x3 lattice (2,048 configurations) whose tables suit profiler
    captures; that is not a bench line."""
    import torch
    from cdet_gb300.integrand import CdetIntegrand
    from cdet_gb300.params import CdetParams, half_lattice_mask
    from cdet_gb300.synthetic import uniform_configurations
    from cdet_gb300.tables import build_tables
    side = 3 if args.stress_small else 12
    params = CdetParams(n1=side, n2=side, beta="10", mu="-0.5", u="6", alpha_up="0", alpha_down="0",
                        mask_sites=half_lattice_mask(side, side), cheb_nu=192, cheb_nv=192)
    default_batch = 2048 if args.stress_small else 8192
    batch, order = args.batch if args.batch != 65536 else default_batch, 14
    t0 = time.perf_counter()
    tables = build_tables(params, device="cuda")
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    torch.cuda.empty_cache()  # the precompute's temporaries; the slices are allocated outside torch
    gpu = CdetIntegrand(params, tables)
    gpu.reserve(batch, order)
    gpu.set_assembly("split")
    t0 = time.perf_counter()
    gpu.prepare_split()
    slice_s = time.perf_counter() - t0
    free_b, total_b = torch.cuda.mem_get_info()
    n_batches = args.steps + args.warmup
    host = [uniform_configurations(20261210 + k, batch, order) for k in range(n_batches)]
    dv = [torch.from_numpy(x).cuda() for x in host]
    o = torch.full((batch,), order, dtype=torch.int32, device="cuda")
    vals = torch.empty(batch, dtype=torch.float64, device="cuda")
    st = torch.empty(batch, dtype=torch.int32, device="cuda")
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.int32, device="cuda")  # 512 MiB > L2
    clocks = ClockSampler(0)
    clocks.start()
    time.sleep(2.0)
    results = {}
    for path in ("fp64", "split"):
        gpu.set_assembly(path)
        for w in range(args.warmup):
            flush.fill_(1)
            gpu.integrand_device(dv[args.steps + w], o, vals, st)
        torch.cuda.synchronize()
        gpu.profile(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for k in range(args.steps):
            flush.fill_(1)
            gpu.integrand_device(dv[k], o, vals, st)
        e1.record()
        torch.cuda.synchronize()
        stage_ms, launches = gpu.profile_read()
        gpu.profile(False)
        results[path] = (e0.elapsed_time(e1), stage_ms, launches, vals.cpu().numpy().copy(), st.cpu().numpy().copy())
        if path == "split":
            split_counters = gpu.split_counters()
    clock_info = clocks.stop()
    # end to end (split) through the host-buffer call
    gpu.set_assembly("split")
    pv = [torch.from_numpy(x).pin_memory() for x in host[:args.steps]]
    po = torch.full((batch,), order, dtype=torch.int32).pin_memory()
    pout = torch.empty(batch, dtype=torch.float64).pin_memory()
    pst = torch.empty(batch, dtype=torch.int32).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        rc = gpu._lib.cdet_integrand_host(gpu._ctx, pv[k].data_ptr(), po.data_ptr(), batch, order,
                                          pout.data_ptr(), pst.data_ptr())
        if rc not in (0, 4):
            raise RuntimeError("host-buffer evaluation failed: " + gpu._lib.cdet_last_error().decode())
    e2e_s = time.perf_counter() - t0
    f_ms, f_stage, f_launch, f_vals, f_st = results["fp64"]
    s_ms, s_stage, s_launch, s_vals, s_st = results["split"]
    ok = (f_vals != 0) & (f_st == 0) & (s_st == 0)
    rel = np.abs(s_vals[ok] - f_vals[ok]) / np.abs(f_vals[ok])
    # Green matrices of both assemblies on a sample of the last batch
    sample = dv[args.steps - 1][:1024].contiguous()
    so = o[:1024].contiguous()
    gpu.set_assembly("fp64")
    g64, _, _ = gpu.assemble(sample, so)
    gpu.set_assembly("split")
    gsp, _, _ = gpu.assemble(sample, so)
    torch.cuda.synchronize()
    gscale = g64.abs().amax(dim=3, keepdim=True).clamp_min(1e-300)
    green_rel = float(((gsp - g64).abs() / gscale).max().item())
    _, bf16_peak, peak_kind = peaks()
    nu, nv = params.cheb_nu, params.cheb_nv
    lookups = batch * 2 * order * order
    assembly_ms = s_stage[1] / args.steps
    achieved = lookups * 2.0 * nu * nv / (assembly_ms / 1e3) / 1e12
    issued_tflops = split_counters[0] * 2.0 * 128 * 16 / (assembly_ms / 1e3) / 1e12

    def per_step(ms):
        return {"split_prep": ms[0] / args.steps, "assembly": ms[1] / args.steps,
                "minors": ms[2] / args.steps, "cdet": ms[3] / args.steps}

    line = {
        "metric": "configs/s at order 14, 12x12 / degree 192 stress: split assembly vs plain FP64",
        "value": batch * args.steps / (s_ms / 1e3), "unit": UNIT, "higher_is_better": True, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": s_ms / args.steps,
        "dtype": "f64 (split fp16-digit tcgen05 assembly, FP64 minors and CDet)",
        "data": "synthetic (seeded uniform vertices, tables from the in-tree precompute)",
        "config": {"workload": f"{side}x{side} Hubbard t=1 U=6 beta=10 mu=-0.5, half-lattice subsystem, "
                               f"Chebyshev degree 192, order n=14, {batch} configurations per step",
                   "lattice": f"{side}x{side}", "U": 6, "beta": 10, "mu": -0.5, "mask": "half lattice x<6",
                   "cheb_degree": 192, "order": order, "batch": batch,
                   "l2": "flushed between steps (512 MiB write)"},
        "e2e": {"value": batch * args.steps / e2e_s, "unit": UNIT,
                "h2d_bytes_per_step": batch * order * 4 * 8 + batch * 4,
                "d2h_bytes_per_step": batch * 8 + batch * 4},
        "gpu_launches": int(s_launch),
        "stages_ms_per_step": per_step(s_stage),
        "roofline": {"kernel": "split_assembly<chunked> (tcgen05 fp16 digit slices, 2 x 2 sub-blocks)",
                     "bound": "tensor", "achieved": achieved, "peak": bf16_peak, "unit": "TFLOP/s",
                     "frac": achieved / bf16_peak, "traffic": None,
                     "peak_source": f"{peak_kind} (MEASURED_PEAKS.json bf16_tflops)",
                     "algorithmic": "lookups x 2 x 192 x 192 (2 sets x n^2 lookups per configuration)",
                     "tcgen05_mma_columns_per_launch": split_counters[0],
                     "tensor_issue_tflops": issued_tflops, "tensor_issue_frac": issued_tflops / bf16_peak,
                     "slice_bytes_streamed_per_launch": split_counters[1]},
        "clocks": clock_info,
        "fp64_path": {"value": batch * args.steps / (f_ms / 1e3), "unit": UNIT, "ms_per_step": f_ms / args.steps,
                      "gpu_launches": int(f_launch), "stages_ms_per_step": per_step(f_stage)},
        "split_over_fp64": f_ms / s_ms,
        "split_vs_fp64_rel_err_order14": {
            "configs": int(ok.sum()), "median": float(np.median(rel)), "p90": float(np.percentile(rel, 90)),
            "max": float(rel.max()),
            "normwise": float(np.abs(s_vals - f_vals).max() / max(np.abs(f_vals).max(), 1e-300)),
            "note": "per-configuration relative error; the FP64 integrand's own round-off floor at order 14 "
                    "(a 1-ulp change of the Green entries moves it by this much)"},
        "green_split_vs_fp64_max_rel": green_rel,
        "derived": derived_rates(batch * args.steps / (s_ms / 1e3), order),
        "flagged_configs": {"fp64": int((f_st != 0).sum()), "split": int((s_st != 0).sum())},
        "setup_s": {"tables": build_s, "slices": slice_s},
        "device_memory_gb": {"used_after_slicing": (total_b - free_b) / 1e9, "total": total_b / 1e9},
        "cpu_baseline": None,
        "cpu_baseline_note": "not timed: the host oracle would need a host copy of the tables (98 GB at 12x12)",
    }
    print(json.dumps(line))
    gpu.close()


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="configurations in the CPU-baseline sample (default 64 per thread)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-precision", action="store_true", help="skip the per-order precision study")
    ap.add_argument("--no-dd", action="store_true", help="skip timing the double-double integrand")
    ap.add_argument("--integrand-form", choices=["auto", "staged", "queue"], default="auto",
                    help="the headline's layout after the assembly: the autotuner's choice (default) or a fixed one")
    ap.add_argument("--precision-configs", type=int, default=512,
                    help="configurations per order in the precision study")
    ap.add_argument("--preset", choices=["8x8-d128", "6x6-d96"], default="8x8-d128",
                    help="6x6-d96 is a smaller case for profiler captures, not a bench line")
    ap.add_argument("--batch", type=int, default=65536, help="configurations per step per GPU")
    ap.add_argument("--path", choices=["both", "split", "fp64"], default="both",
                    help="both: time the FP64 form and the split form, report the split form")
    ap.add_argument("--mcmcmc", action="store_true",
                    help="time the device MCMCMC chains instead (a separate line, not the headline)")
    ap.add_argument("--chains", type=int, default=128, help="chains for --mcmcmc")
    ap.add_argument("--mixed", action="store_true",
                    help="time a batch of mixed orders 1..10 (a separate line, not the headline)")
    ap.add_argument("--mcmcmc-steps", type=int, default=2000, help="timed production steps for --mcmcmc")
    ap.add_argument("--stress", action="store_true",
                    help="time the 12x12 / degree-192 / order-14 stress case (a separate line, not the headline)")
    ap.add_argument("--stress-small", action="store_true",
                    help="with --stress: a 3x3 lattice and 2,048 configurations, for profiler captures")
    args = ap.parse_args()
    global PRESET, BATCH
    PRESET, BATCH = args.preset, args.batch
    args.warmup = max(args.warmup, 3)  # at least three untimed warm-up steps
    if args.mixed:
        run_mixed(args)
        return
    if args.stress:
        run_stress(args)
        return
    if args.mcmcmc:
        run_mcmcmc(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
