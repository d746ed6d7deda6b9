#!/usr/bin/env python3
"""Benchmark of the proving hot path on GB300: committed + sumchecked field elements per second.

Workload (one step): the 256-polynomial commitment, 256 rows of k = 2^20 uniform Goldilocks
values encoded at rate 1/2 (n = 2^21), absorbed into 2^21 column chains in blocks of B = 32 rows
and merkled into a root; then a degree-3 sumcheck of Σ f·g·h over three tables of 2^22 values
with challenges from the BLAKE3 transcript. Units per step: 2^28 committed elements plus
3·2^22 sumchecked table entries. Inputs are SplitMix64 streams (seeded synthetic data).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`value` times K steps with every input already in HBM (CUDA events on the library's stream);
`e2e` times the same steps through the host-memory API, the host-to-device copy of the inputs
from pinned memory and the read-back of the root and proof inside. The reference arm times the
CPU port of the reference's algorithms (the plain-C oracle) on this host's cores.
Multi-GPU: one independent replica per GPU (the path needs no exchange), weak scaling.
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

from tessera_gb300.workloads import splitmix_words  # noqa: E402  (numpy only; loads no native code)

NPOLYS, LOG_K, LOG_R, ROW_BLOCK = 256, 20, 1, 32
SC_VARS, SC_DEGREE = 22, 3
SEED = 0x00650002
COMMITTED = NPOLYS << LOG_K
SUMCHECKED = SC_DEGREE << SC_VARS
UNITS = COMMITTED + SUMCHECKED
CONFIG = {
    "workload": "commit 256 x 2^20 Goldilocks at rate 1/2 (n = 2^21, B = 32, BLAKE3 column chains + Merkle root) "
                "+ degree-3 sumcheck of f*g*h over 3 x 2^22",
    "polys": NPOLYS, "log_k": LOG_K, "log_inv_rate": LOG_R, "row_block": ROW_BLOCK,
    "sumcheck_vars": SC_VARS, "sumcheck_degree": SC_DEGREE,
    "l2": "inputs larger than L2 (2 GiB rows, 4 GiB codewords per step)",
    "data": "SplitMix64 uniform Goldilocks",
}
MASK64 = (1 << 64) - 1
P = 0xFFFFFFFF00000001


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons every 200 ms; begin()/end() mark the timed
    region on the host clock, and the summary keeps the samples that arrived inside it (started
    before the warm-up, so that the sampler is running when the region starts)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.rows, self.proc = index, [], None
        self.t0 = self.t1 = None

    def begin(self):
        self.t0 = time.time()

    def end(self):
        self.t1 = time.time()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([time.time()] + [x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        inside = [r[1:] for r in self.rows if self.t0 is None or self.t0 <= r[0] <= (self.t1 or r[0]) + 0.05]
        rows = inside or [r[1:] for r in self.rows]  # a region shorter than the sampling period
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 5 + i and r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside)}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, world: int, device) -> float:
    """The largest of every rank's value through the process group (the whole job's time is the
    slowest rank's); the value itself with one rank."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, world: int, ms: float) -> float:
    """Whole-job throughput: every rank's units over the slowest rank's time (ms)."""
    return units_per_rank * world / (ms / 1e3)


# ---- CPU port (the reference arm and the cpu_baseline leg) ---------------------------------------

class CpuStep:
    """The CPU port's time for one full step of the workload, composed from timed components.

    A full step at 1 thread takes about a minute, so each run times bounded samples of every
    component and scales each by the units it processed: `polys` of the 256 rows encoded (k = 2^20,
    rate 1/2), the 2^21 column chains' init and one 32-row absorb block over 2^21 >> col_shift
    columns, the Merkle tree over as many leaves, and the whole degree-3 sumcheck over 3 x 2^22.
    step = 256/polys · encode + 2^col_shift · (init + 8 · block + merkle) + sumcheck, each a
    linear cost in its units (rows, columns, blocks, nodes)."""

    def __init__(self, threads: int, polys: int, col_shift: int):
        from oracle import oracle as O

        self.O, self.threads, self.polys, self.col_shift = O, threads, polys, col_shift
        n = 1 << (LOG_K + LOG_R)
        self.cols = n >> col_shift
        self.rows = O.splitmix(SEED, polys << LOG_K)
        self.block = O.splitmix(SEED + 7, ROW_BLOCK * self.cols)  # symbols of one absorb block
        self.leaves = np.frombuffer(O.splitmix(SEED + 8, 4 * self.cols).tobytes(), dtype=np.uint8).reshape(-1, 32)
        self.tabs = [O.splitmix(SEED + 1 + i, 1 << SC_VARS) for i in range(3)]
        self.ctx = bench_context().tce()

    def run(self) -> dict:
        O, T = self.O, self.threads
        cid = bytes([0x65]) * 32
        t0 = time.perf_counter()
        O.encode_rows(self.rows, LOG_K, LOG_R, threads=T)
        t1 = time.perf_counter()
        O.column_chains(cid, self.block[:0], self.cols, ROW_BLOCK, threads=T)  # init only
        t2 = time.perf_counter()
        O.column_chains(cid, self.block, self.cols, ROW_BLOCK, threads=T)  # init + one block
        t3 = time.perf_counter()
        O.merkle_tree(self.leaves, threads=T)
        t4 = time.perf_counter()
        O.prove_batch(O.OracleTranscript(self.ctx), "stage/0", SC_DEGREE, [[(x, False, False) for x in self.tabs]])
        t5 = time.perf_counter()
        scale = 1 << self.col_shift
        blocks = NPOLYS // ROW_BLOCK
        parts = {"encode_s": (t1 - t0) * NPOLYS / self.polys, "chain_init_s": (t2 - t1) * scale,
                 "chain_blocks_s": max(0.0, (t3 - t2) - (t2 - t1)) * scale * blocks, "merkle_s": (t4 - t3) * scale,
                 "sumcheck_s": t5 - t4}
        parts["step_s"] = sum(parts.values())
        parts["sampled_s"] = t5 - t0
        return parts

    def sample(self) -> str:
        return (f"composed step: {self.polys} of 256 rows encoded, chains (init + one 32-row block) and the Merkle "
                f"tree over 2^{LOG_K + LOG_R - self.col_shift} of 2^{LOG_K + LOG_R} columns, each scaled to the full "
                f"step, plus the whole sumcheck over 3 x 2^{SC_VARS}; {self.threads} thread(s)")


def rfc0020(step: CpuStep, warmup: int, runs: int) -> dict:
    """Warm-up runs, then measured runs: median, min, max and CV of the composed step time (the
    reference's benchmarking protocol, docs/perf/README.md:25-27, flags CV above 3 %)."""
    for _ in range(warmup):
        step.run()
    rs = [step.run() for _ in range(runs)]
    ts = [r["step_s"] for r in rs]
    med = statistics.median(ts)
    cv = statistics.pstdev(ts) / statistics.mean(ts) if len(ts) > 1 else 0.0
    mid = rs[ts.index(sorted(ts)[len(ts) // 2])]
    return {"step_s_median": med, "step_s_min": min(ts), "step_s_max": max(ts), "cv": cv, "noisy": cv > 0.03,
            "warmup": warmup, "runs": runs, "threads": step.threads, "value": UNITS / med,
            "components_s": {k: v for k, v in mid.items() if k not in ("step_s", "sampled_s")},
            "sampled_s_per_run": statistics.mean(r["sampled_s"] for r in rs), "sample": step.sample()}


def bench_context():
    from tessera_gb300.hash import Mode, SessionContext

    return SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([0x65]) * 32, bytes([0x65]) * 16)


def run_reference(args) -> None:
    """The reference arm: the CPU port of the reference's algorithms (the oracle) on this host's
    cores, one full step of the workload composed from timed components (CpuStep) per run, at
    all host threads (the value) and at one thread (the reference's default), each with the
    warm-up and measured runs of the reference's benchmarking protocol."""
    world, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O

    O.build()
    threads = O.threads_available()
    allc = rfc0020(CpuStep(threads, args.ref_polys, 0), max(3, args.warmup), args.steps)
    one = rfc0020(CpuStep(1, 2, 4), 1, 3)
    value = allc["value"]
    line = {
        "metric": "committed+sumchecked field elems/s", "value": value, "unit": "elems/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": 1e3 * allc["step_s_median"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (Goldilocks)",
        "data": "synthetic", "impl": "reference", "config": CONFIG,
        "composed": "each step's time is composed from timed samples of every component, scaled to the full "
                    "256 x 2^20 commitment and 3 x 2^22 sumcheck (a full step at one thread takes about a minute)",
        "cpu_baseline": {"value": value, "unit": "elems/s", "cores": threads, "kind": "port", "sample": allc["sample"],
                         "all_cores": allc, "one_thread": one},
        "e2e": {"value": value, "unit": "elems/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "latency_ms": {"p50": 1e3 * allc["step_s_median"], "p99": 1e3 * allc["step_s_max"]},
    }
    print(json.dumps(line), flush=True)


# ---- GPU arm ------------------------------------------------------------------------------------

def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def bind_gpu_local_cpus(ordinal: int) -> dict | None:
    """Restricts this process to the CPUs local to the GPU (its PCI device's local_cpulist), so
    that host buffers allocated and touched next land on the GPU's NUMA node; returns what was
    found, or None where the topology is not visible."""
    try:
        import torch

        p = torch.cuda.get_device_properties(ordinal)
        dev = Path(f"/sys/bus/pci/devices/{p.pci_domain_id:04x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0")
        node = int((dev / "numa_node").read_text().strip())
        cpus = set()
        for part in (dev / "local_cpulist").read_text().strip().split(","):
            if part:
                a, _, b = part.partition("-")
                cpus.update(range(int(a), int(b or a) + 1))
        cpus &= os.sched_getaffinity(0)
        if not cpus:
            return None
        os.sched_setaffinity(0, cpus)
        return {"numa_node": node, "local_cpus": len(cpus)}
    except Exception:  # noqa: BLE001 - no sysfs, no affinity API, or a device without topology
        return None


def traffic_table() -> dict:
    p = ROOT / "profiles" / "traffic.json"
    return json.loads(p.read_text()) if p.exists() else {}


def run_gpu(args) -> None:
    import ctypes

    import torch

    from tessera_gb300 import _native as N
    from tessera_gb300.device import Device
    from tessera_gb300.hash import Transcript
    from tessera_gb300.sumcheck import Instance, Protocol, Table, prove_batch

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    dev = Device(local, lde_group_bytes=args.lde_group_mib << 20)
    cuda = f"cuda:{local}"
    stream = torch.cuda.ExternalStream(dev.stream_ptr(), device=cuda)

    # inputs: host (pinned, for e2e) and resident device copies; the pinned pages are first
    # touched from the GPU's own NUMA node, where its host link is shortest
    saved = os.sched_getaffinity(0) if hasattr(os, "sched_getaffinity") else None
    host_numa = bind_gpu_local_cpus(local)
    rows_h = torch.from_numpy(splitmix_words(SEED, COMMITTED).view(np.int64)).pin_memory()
    tabs_h = [torch.from_numpy(splitmix_words(SEED + 1 + i, 1 << SC_VARS).view(np.int64)).pin_memory() for i in range(3)]
    if saved is not None and host_numa:
        os.sched_setaffinity(0, saved)
    rows_d = rows_h.to(cuda)
    tabs_d = [t.to(cuda) for t in tabs_h]
    n = 1 << (LOG_K + LOG_R)
    npolys = COMMITTED >> LOG_K
    cw_d = torch.empty(npolys * n, dtype=torch.int64, device=cuda)
    nodes_d = torch.empty((2 * n - 1) * 32, dtype=torch.uint8, device=cuda)
    # the host-buffer path reads the pinned words in place (uint64 views, no host copies)
    rows_hw = rows_h.numpy().view(np.uint64)
    tabs_hw = [t.numpy().view(np.uint64) for t in tabs_h]
    torch.cuda.synchronize()
    cid = (ctypes.c_uint8 * 32)(*([0x65] * 32))
    root = ctypes.create_string_buffer(32)

    def commit(src):
        N.call("tg_commit_unmasked_dev", dev.handle, LOG_K, LOG_R, ROW_BLOCK, cid, ctypes.c_void_p(src.data_ptr()), npolys,
               ctypes.c_void_p(cw_d.data_ptr()), ctypes.c_void_p(nodes_d.data_ptr()), root, None)

    def sumcheck(tabs):
        t = Transcript(bench_context())
        return prove_batch(t, Protocol.ONE, "stage/0", SC_DEGREE, [Instance([Table.base(x) for x in tabs])], device=dev)

    def step():
        commit(rows_d)
        return sumcheck(tabs_d)

    def step_e2e():
        # the C ABI's host-buffer calls: rows and tables from pinned host memory, the root and the
        # proof back to the host (the library overlaps the row copies with the encoder)
        N.call("tg_commit_unmasked", dev.handle, LOG_K, LOG_R, ROW_BLOCK, cid, ctypes.c_void_p(rows_hw.ctypes.data),
               npolys, None, root)
        return sumcheck(tabs_hw)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    clocks = Clocks(local).__enter__()  # sampling from the warm-up on; the summary keeps the timed region's
    try:
        for _ in range(args.warmup):
            step()
        barrier()
        int_peaks = dev.int_peaks()  # register-only microbenchmarks, outside the timed region

        # the timed region: K steps, inputs resident
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
        launches0 = dev.launches()
        dev.profile(True)
        torch.cuda.synchronize()
        clocks.begin()
        ev[0].record(stream)
        for i in range(args.steps):
            step()
            ev[i + 1].record(stream)
        stream.synchronize()
        clocks.end()
    finally:
        clocks.__exit__(None, None, None)
    dev.profile(False)
    prof = dev.profile_read()
    launches = dev.launches() - launches0
    barrier()
    step_ms = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    total_ms = max_over_ranks(ev[0].elapsed_time(ev[-1]), world, cuda)
    ms_per_step = total_ms / args.steps
    value = job_rate(UNITS, world, ms_per_step)

    # the host link's rate from pinned memory (the best of three 512 MiB copies), which bounds the
    # end-to-end step from below: it moves h2d bytes per step
    link = rows_h[: 64 << 20]
    link_d = torch.empty_like(link, device=cuda)
    link_gbs = 0.0
    for _ in range(3):
        l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0.record(stream)
        with torch.cuda.stream(stream):
            link_d.copy_(link, non_blocking=True)
        l1.record(stream)
        l1.synchronize()
        link_gbs = max(link_gbs, link.numel() * 8 / (l0.elapsed_time(l1) / 1e3) / 1e9)
    del link_d

    # end to end through the host-memory path
    for _ in range(max(1, args.warmup // 2)):
        step_e2e()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step_e2e()
    e1.record(stream)
    stream.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, cuda)
    h2d = COMMITTED * 8 + 3 * (1 << SC_VARS) * 8
    d2h = 32 + SC_VARS * SC_DEGREE * 16 + 3 * 16
    # Release torch's buffers while the library's stream (which their copies used) still exists,
    # and return torch's cached pinned blocks while the context is certainly alive.
    stream.synchronize()
    del rows_hw, tabs_hw, rows_h, tabs_h, rows_d, tabs_d, cw_d, nodes_d, link
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    if hasattr(torch._C, "_host_emptyCache"):
        torch._C._host_emptyCache()
    dev.close()

    if rank != 0:
        return
    # roofline of the dominant kernel: the encoder (its passes run back to back over one launch
    # group of rows) against HBM; algorithmic bytes = each row read once + its codeword written once
    kernels = {k: {"ms_per_step": v[0] / args.steps, "launches_per_step": v[1] / args.steps,
                   "share": v[0] / max(1e-9, sum(x[0] for x in prof.values()))} for k, v in prof.items()}
    lde_names = sorted(k for k in prof if k.startswith("lde_"))
    lde_ms = sum(prof[k][0] for k in lde_names)
    lde_launch_groups = prof.get("lde_pass_a", (0, 1, 0))[1]
    rows_done = prof.get("lde_pass_a", (0, 0, 0))[2]
    bytes_per_row = 8 * (1 << LOG_K) + 8 * (1 << (LOG_K + LOG_R))
    peaks = measured_peaks()
    achieved = (bytes_per_row * rows_done) / (lde_ms / 1e3) / 1e9 if lde_ms else None
    traffic = traffic_table().get("lde_dram_bytes_per_row")
    rows_per_group = rows_done / max(1, lde_launch_groups)
    roofline = {
        "kernel": "lde encoder (" + "+".join(lde_names) + "; one launch = one group of rows through all passes)",
        "bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
        "frac": (achieved / peaks["hbm_gbs"]) if achieved else None, "peak_source": peaks["source"],
        "algorithmic_bytes_per_row": bytes_per_row, "rows_per_launch": rows_per_group,
        "traffic": (traffic * rows_per_group) if traffic else None,
        "traffic_unit": "DRAM bytes per launch (all passes, ncu, scaled by rows)",
        "traffic_source": ("profiles/traffic.json, captured at commit " + traffic_table().get("captured_at_commit", "?"))
                          if traffic else None,
        "note": "the encoder is bound by the integer pipes, not by HBM; int_rate gives its fraction of the measured integer peak",
    }
    butterflies_per_row = ((1 << LOG_K) // 2) * LOG_K + ((1 << (LOG_K + LOG_R)) // 2) * (LOG_K + LOG_R)
    bf_rate = butterflies_per_row * rows_done / (lde_ms / 1e3) if lde_ms else None
    # BLAKE3 in the column chains: one compression per 64-byte block of each step's 32 + 8·b bytes
    n_cols = 1 << (LOG_K + LOG_R)
    blocks = [min(ROW_BLOCK, npolys - r0) for r0 in range(0, npolys, ROW_BLOCK)]
    comp_per_step = n_cols * sum((32 + 8 * b + 63) // 64 for b in blocks)
    absorb_ms = prof.get("column_absorb", (0, 0, 0))[0] / args.steps
    comp_rate = comp_per_step / (absorb_ms / 1e3) if absorb_ms else None
    int_rate = {
        "lde": {"achieved": bf_rate, "peak": int_peaks["butterflies_per_s"], "unit": "radix-2 butterflies/s",
                "frac": bf_rate / int_peaks["butterflies_per_s"] if bf_rate else None,
                "radix2_butterflies_per_row": butterflies_per_row,
                "note": "peak = the same lazy shift-twiddle butterflies in registers only (tg_measure_int_peaks); "
                        "the encoder also pays one to three general products per element per pass"},
        "column_absorb": {"achieved": comp_rate, "peak": int_peaks["blake3_compressions_per_s"],
                          "unit": "BLAKE3 compressions/s",
                          "frac": comp_rate / int_peaks["blake3_compressions_per_s"] if comp_rate else None,
                          "compressions_per_step": comp_per_step},
        "measured_peaks": int_peaks,
    }

    line = {
        "metric": "committed+sumchecked field elems/s", "value": value, "unit": "elems/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64 (Goldilocks)", "data": "synthetic", "config": CONFIG,
        "e2e": {"value": job_rate(UNITS, world, e2e_ms), "unit": "elems/s", "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "host_link_gbs": link_gbs, "host_link_floor_ms": h2d / (link_gbs * 1e9) * 1e3 if link_gbs else None,
                "note": "the step's copies cross the host link at host_link_gbs (measured here, pinned memory); "
                        "e2e is at least max(ms_per_step, host_link_floor_ms)"},
        "latency_ms": {"p50": statistics.median(step_ms), "p99": max(step_ms) if len(step_ms) < 100 else
                       sorted(step_ms)[int(0.99 * len(step_ms))]},
        "gpu_launches": launches,
        "host_buffers": host_numa or "NUMA placement not visible; pinned with default first-touch",
        "roofline": roofline,
        "int_rate": int_rate,
        "kernels": kernels,
        "clocks": clocks.summary(),
    }
    if not args.no_cpu_baseline and world == 1:
        from oracle import oracle as O

        O.build()
        threads = O.threads_available()
        allc = rfc0020(CpuStep(threads, args.cpu_polys, 0), 1, 5)
        one = rfc0020(CpuStep(1, 2, 4), 1, 3)
        line["cpu_baseline"] = {"value": allc["value"], "unit": "elems/s", "cores": threads, "kind": "port",
                                "sample": allc["sample"], "all_cores": allc, "one_thread": one}
    print(json.dumps(line), flush=True)


SEED_BATCHED = 0x00650003


def run_batched(args) -> None:
    """The batched workload (64 uneven commitments + 64 uneven sumchecks, one transcript each),
    batched (a CUDA-graph commit plan with autotuned streams + one prove_many) against the plain
    path (one commit_unmasked_dev and one prove_batch per request, in turn), on the same device
    buffers. Prints one JSON line with both; per-request latency is the time from the batch's start
    to that request's result."""
    import ctypes

    import torch

    from tessera_gb300 import _native as N
    from tessera_gb300.device import Device
    from tessera_gb300.hash import Mode, SessionContext, Transcript
    from tessera_gb300.pcs import CommitmentParams, CommitPlan
    from tessera_gb300.sumcheck import Instance, Protocol, Table, prove_batch, prove_many
    from tessera_gb300.workloads import batched, fill_device

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    cuda = f"cuda:{local}"
    dev = Device(local)
    cs, ss = batched(SEED_BATCHED)
    rows = [fill_device(torch.empty(c.polys << c.log_k, dtype=torch.int64, device=cuda), c.seed, dev) for c in cs]
    tabs = [[fill_device(torch.empty(1 << s.vars, dtype=torch.int64, device=cuda), s.seed + i, dev)
             for i in range(s.degree)] for s in ss]
    params = [CommitmentParams(c.log_k, c.log_inv_rate, 0, ROW_BLOCK, c.commitment_id) for c in cs]
    t0 = time.perf_counter()
    plan = CommitPlan(params, rows, device=dev)
    plan_s = time.perf_counter() - t0
    committed = sum(c.polys << c.log_k for c in cs)
    sumchecked = sum(s.degree << s.vars for s in ss)
    units = committed + sumchecked

    def ctx(s):
        return SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([0x65]) * 32,
                              s.session_id)

    def batched_step(lat):
        start = time.perf_counter()
        plan.launch()
        prove_many([(Transcript(ctx(s)), Protocol.ONE, "stage/0", s.degree, [Instance([Table.base(x) for x in t])])
                    for s, t in zip(ss, tabs)], device=dev)
        lat.extend([time.perf_counter() - start] * (len(cs) + len(ss)))

    def plain_step(lat):
        start = time.perf_counter()
        root = ctypes.create_string_buffer(32)
        for p, r, c in zip(params, rows, plan.commitments):
            N.call("tg_commit_unmasked_dev", dev.handle, p.log2_k, p.log2_inv_rate, p.row_block,
                   (ctypes.c_uint8 * 32)(*p.commitment_id), ctypes.c_void_p(r.data_ptr()), r.numel() >> p.log2_k,
                   ctypes.c_void_p(c.codewords.data_ptr()), ctypes.c_void_p(c.nodes.data_ptr()), root, None)
            lat.append(time.perf_counter() - start)
        for s, t in zip(ss, tabs):
            prove_batch(Transcript(ctx(s)), Protocol.ONE, "stage/0", s.degree, [Instance([Table.base(x) for x in t])],
                        device=dev)
            lat.append(time.perf_counter() - start)

    out = {}
    for name, fn in (("plain", plain_step), ("batched", batched_step)):
        for _ in range(args.warmup):
            fn([])
        torch.cuda.synchronize()
        lat, times = [], []
        l0 = dev.launches()
        for _ in range(args.steps):
            a = time.perf_counter()
            fn(lat)
            times.append(time.perf_counter() - a)
        launches = (dev.launches() - l0) / args.steps
        lat_ms = sorted(x * 1e3 for x in lat)
        ms = 1e3 * sum(times) / len(times)
        out[name] = {"value": units / (ms / 1e3), "ms_per_step": ms,
                     "latency_ms": {"p50": statistics.median(lat_ms), "p99": lat_ms[int(0.99 * (len(lat_ms) - 1))]},
                     "gpu_launches_per_step": launches}
    info = plan.info()
    plan.close()
    del rows, tabs
    torch.cuda.synchronize()
    dev.close()
    if rank != 0:
        return
    line = {
        "metric": "committed+sumchecked field elems/s; p50/p99 proof latency, batched vs plain",
        "value": out["batched"]["value"], "unit": "elems/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": out["batched"]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64 (Goldilocks)", "data": "synthetic",
        "config": {"workload": "batched: 64 commitments (k = 2^10..2^20 log-uniform, 8/32/128/512 rows, rate 1/2 or "
                               "1/4, B = 32) + 64 sumchecks (10..22 variables, degree 2 or 3, own transcripts)",
                   "seed": SEED_BATCHED, "committed_elems": committed, "sumchecked_elems": sumchecked,
                   "timing": "host wall clock around each step (each step ends with its results on the host)"},
        "batched": out["batched"], "plain": out["plain"],
        "speedup_batched_over_plain": out["plain"]["ms_per_step"] / out["batched"]["ms_per_step"],
        "plan": {**info, "create_s": plan_s},
    }
    print(json.dumps(line), flush=True)


def run_serve(args) -> None:
    """Serving: a Poisson stream of proof requests (commitment + sumcheck units of uneven sizes,
    each on its own transcript) through the proof server (continuous batching, HBM-budget
    admission) against the plain path (one request at a time, in arrival order). Latency is
    arrival to result; a second pass offers every request at once to measure saturated proofs/s."""
    import random

    import torch

    from tessera_gb300.device import Device
    from tessera_gb300.hash import Mode, SessionContext, Transcript
    from tessera_gb300.pcs import CommitmentParams
    from tessera_gb300.serve import ProofRequest, ProofServer, prove_plain

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = Device(local)
    rs = random.Random(SEED_SERVE)
    reqs, arrivals, units, sizes = [], [], 0, []
    t = 0.0
    keep = []
    shapes = []
    for i in range(args.requests):
        if i < args.distinct:  # a new input set; later requests take input set i mod distinct again
            log_k, polys, log_r = rs.randint(10, 16), rs.choice([8, 32, 128]), rs.choice([1, 2])
            vars_, degree = rs.randint(10, 18), rs.choice([2, 3])
            rows = torch.from_numpy(splitmix_words(SEED_SERVE + 2 * i, polys << log_k).view(np.int64)).pin_memory()
            tabs = [torch.from_numpy(splitmix_words(SEED_SERVE + 7919 * i + k, 1 << vars_).view(np.int64)).pin_memory()
                    for k in range(degree)]
            keep.append((rows, tabs))
            shapes.append((log_k, polys, log_r, vars_, degree))
        log_k, polys, log_r, vars_, degree = shapes[i % args.distinct]
        rows, tabs = keep[i % args.distinct]
        ctx = SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([0x65]) * 32,
                             i.to_bytes(16, "little"))
        cid = bytes(rs.randrange(256) for _ in range(32))
        reqs.append(ProofRequest(CommitmentParams(log_k, log_r, 0, ROW_BLOCK, cid), rows.numpy().view(np.uint64),
                                 degree, [x.numpy().view(np.uint64) for x in tabs], Transcript(ctx), "stage/0",
                                 args.queries))
        units += (polys << log_k) + (degree << vars_)
        sizes.append((polys << log_k) + (degree << vars_))
        t += rs.expovariate(args.rate)
        arrivals.append(t)

    def plain(offered):
        lat = []
        start = time.perf_counter()
        for r, a in zip(reqs, offered):
            now = time.perf_counter() - start
            if a > now:
                time.sleep(a - now)
            prove_plain(r, dev)
            lat.append(time.perf_counter() - start - a)
        return time.perf_counter() - start, lat

    def served(offered):
        with ProofServer(dev, hbm_budget_bytes=args.serve_budget_gib << 30, slots=args.slots) as srv:
            tickets = [None] * len(reqs)
            start = time.perf_counter()

            def producer():
                for i, (r, a) in enumerate(zip(reqs, offered)):
                    now = time.perf_counter() - start
                    if a > now:
                        time.sleep(a - now)
                    tickets[i] = srv.submit(r)

            th = threading.Thread(target=producer)
            th.start()
            th.join()
            res = [srv.wait(tk) for tk in tickets]
            wall = time.perf_counter() - start
            st = srv.stats()
        st["stages"] = [(round(x.queued_ms, 3),) + tuple(round(v, 3) for v in x.stage_ms) for x in res]
        return wall, [x.latency_ms / 1e3 for x in res], st

    # warm-up: shapes' tables, pools, pinned paths
    for r in reqs[: min(8, len(reqs))]:
        prove_plain(r, dev)
    served([0.0] * len(reqs))
    out = {}
    for mode, offered in (("poisson", arrivals), ("saturated", [0.0] * len(reqs))):
        pw, pl = plain(offered)
        sw, sl, st = served(offered)
        q = lambda xs, f: sorted(xs)[min(len(xs) - 1, int(f * len(xs)))] * 1e3  # noqa: E731

        def tail(xs):  # the slowest requests: (latency ms, request index, committed + sumchecked elements)
            worst = sorted(range(len(xs)), key=lambda i: -xs[i])[:4]
            return [(round(xs[i] * 1e3, 3), i, sizes[i]) for i in worst]

        out[mode] = {
            "plain": {"proofs_per_s": len(reqs) / pw, "elems_per_s": units / pw,
                      "latency_ms": {"p50": q(pl, 0.5), "p99": q(pl, 0.99)}, "slowest": tail(pl)},
            "served": {"proofs_per_s": len(reqs) / sw, "elems_per_s": units / sw,
                       "latency_ms": {"p50": q(sl, 0.5), "p99": q(sl, 0.99)}, "slowest": tail(sl),
                       "slowest_stages_ms": [st["stages"][i] for _, i, _ in tail(sl)],
                       # each stage's own time (admission wait, commit, sumcheck, opening), p50 and p99
                       "stage_ms": {name: {"p50": q([x / 1e3 for x in ds], 0.5), "p99": q([x / 1e3 for x in ds], 0.99)}
                                    for name, ds in zip(("queued", "commit", "sumcheck", "opening"),
                                                        zip(*[(g[0], g[1] - g[0], g[2] - g[1], g[3] - g[2])
                                                              for g in st["stages"] if len(g) == 4]))},
                       "peak_inflight": st["peak_inflight"], "peak_gib": st["peak_bytes"] / 2**30},
        }
    del keep
    dev.close()
    if rank != 0:
        return
    sat = out["saturated"]
    line = {
        "metric": "proofs/s and committed+sumchecked elems/s; p50/p99 proof latency, served vs plain",
        "value": sat["served"]["proofs_per_s"], "unit": "proofs/s", "n_gpus": world, "steps": 1, "warmup": 1,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (Goldilocks)", "data": "synthetic",
        "config": {"workload": f"serve: {len(reqs)} proof requests (commit 8/32/128 x 2^10..2^16 at rate 1/2 or 1/4, "
                               f"B = 32, then a degree-2/3 sumcheck over 2^10..2^18 bound to the root, then "
                               f"{args.queries} column queries answered from the resident commitment; request i proves input set "
                               f"i mod {min(args.distinct, len(reqs))} on its own transcript), Poisson "
                               f"{args.rate} req/s, then all at once", "seed": SEED_SERVE, "slots": args.slots,
                   "queries": args.queries,
                   "hbm_budget_gib": args.serve_budget_gib, "elems": units,
                   "timing": "host wall clock; latency = arrival to result on the host"},
        **out,
    }
    print(json.dumps(line), flush=True)


# The reference benchmark's c_ℓ inputs (crates/tessera-bench/examples/gpu_unit_costs.rs `l`): fixed
# α and β, and the counter generator's seeds of the lookup tree's keys and values and of the table
# tree's keys, values and multiplicities.
LOGUP_ALPHA = (0x123456789ABCDEF0, 0x0FEDCBA987654321)
LOGUP_BETA = (0x1111222233334444, 0x5555666677778888)
LOGUP_LOOKUP = (1 << 56, 1 << 57, None)
LOGUP_TABLE = (1 << 58, 1 << 59, 1 << 60)


def bench_transcript_context():
    """The reference benchmark's transcript context for its tree proofs (gpu_unit_costs.rs
    transcript()): params "bench/1", statement [0x65; 32], session [0x13; 16]."""
    from tessera_gb300.hash import Mode, SessionContext

    return SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "bench/1", bytes([0x65]) * 32, bytes([0x13]) * 16)


def run_logup(args) -> None:
    """LogUp fraction trees, the reference benchmark's c_ℓ measurement: a lookup tree of 2^A
    generated leaves (1, α − (k + β·v)) and a table tree of 2^T leaves (−m, α − (k + β·v)), each
    built on the device and proven level by level as its own leaf stage on a fresh transcript,
    with the reference benchmark's seeds, α, β and transcript; the time per lookup is the two
    trees' time over 2^A. --impl refgpu runs the reference's own kernels the same way
    (oracle/refgpu.cpp) after checking that both prove each tree to the same transcript."""
    import ctypes

    import torch

    from tessera_gb300.device import Device
    from tessera_gb300.hash import Transcript
    from tessera_gb300.trees import LeafStage, generated_fraction

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = Device(local)
    ctx = bench_transcript_context()

    def one(height, seeds, keep=None):
        start = time.perf_counter()
        t = Transcript(ctx)
        tree = generated_fraction(height, seeds[0], seeds[1], seeds[2], LOGUP_ALPHA, LOGUP_BETA, dev, deferred=True)
        with LeafStage([tree], dev) as st:
            st.prove(t)
        torch.cuda.synchronize()
        if keep is not None:
            keep.append((t.state, t.counter))
        return time.perf_counter() - start

    if args.impl == "refgpu":
        ours = []
        one(args.lookups_log, LOGUP_LOOKUP, ours)
        one(args.rows_log, LOGUP_TABLE, ours)
        torch.cuda.synchronize()
        dev.trim()
        dev.close()
        trees_fb = ROOT / "oracle" / "_ref" / "trees.fatbin"
        lib_path = ROOT / "oracle" / "_build" / "librefgpu.so"
        if not (trees_fb.exists() and lib_path.exists()):
            if rank == 0:
                print(json.dumps({"impl": "refgpu", "unavailable": "the reference kernels were not compiled here "
                                  "(oracle/_ref/trees.fatbin needs the reference checkout)"}))
            return
        lib = ctypes.CDLL(str(lib_path))
        lib.refgpu_last_error.restype = ctypes.c_char_p
        med, same = {}, []
        for name, height, seeds, theirs_ours in (("lookup", args.lookups_log, LOGUP_LOOKUP, ours[0]),
                                                 ("table", args.rows_log, LOGUP_TABLE, ours[1])):
            words = (ctypes.c_uint64 * 7)(seeds[0], seeds[1], seeds[2] or 0, *LOGUP_ALPHA, *LOGUP_BETA)
            out = (ctypes.c_double * 1)()
            state = ctypes.create_string_buffer(32)
            counter = ctypes.c_uint64()
            rc = lib.refgpu_fraction(str(trees_fb).encode(), ctypes.c_uint32(height), words,
                                     ctypes.c_uint32(int(seeds[2] is None)), ctypes.c_int(args.warmup),
                                     ctypes.c_int(args.steps), out, state, ctypes.byref(counter))
            if rc != 0:
                raise RuntimeError("reference kernels: " + lib.refgpu_last_error().decode())
            med[name] = out[0]
            same.append((state.raw, counter.value) == theirs_ours)
        if rank != 0:
            return
        print(json.dumps({
            "metric": "LogUp ps per lookup (fraction-tree build + level sumchecks, lookup and table trees)",
            "value": (med["lookup"] + med["table"]) / (1 << args.lookups_log) * 1e12, "unit": "ps/lookup",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64 (Goldilocks Fp2)", "impl": "refgpu",
            "data": "synthetic (the reference benchmark's counter-generated keys, values and multiplicities)",
            "config": {"workload": f"2^{args.lookups_log} lookups into 2^{args.rows_log} rows, each tree its own proof",
                       "timing": "host wall clock per tree, median over steps, leaves generated on the device inside"},
            "lookup_tree_ms": med["lookup"] * 1e3, "table_tree_ms": med["table"] * 1e3,
            "kernels": "the reference's crates/tessera-gpu/kernels/trees.cu (frac_level_leaves, frac_level, "
                       "frac_sums_*, frac_bind_sums_*, frac_first_*, frac_last_*, eq_table, reduce_sums) compiled "
                       "for sm_103 with its own flags, driven as crates/tessera-gpu/src/fraction.rs "
                       "prove_fraction_tree_in does",
            "final_transcripts_equal_library": same,
        }), flush=True)
        return

    for _ in range(args.warmup):
        one(args.lookups_log, LOGUP_LOOKUP)
        one(args.rows_log, LOGUP_TABLE)
    times = {"lookup": [], "table": []}
    for _ in range(args.steps):  # timed without per-launch events
        times["lookup"].append(one(args.lookups_log, LOGUP_LOOKUP))
        times["table"].append(one(args.rows_log, LOGUP_TABLE))
    dev.profile(True)  # one more step, profiled, for the kernel breakdown
    one(args.lookups_log, LOGUP_LOOKUP)
    one(args.rows_log, LOGUP_TABLE)
    dev.profile(False)
    prof = dev.profile_read()
    kernels = {k: {"ms_per_step": v[0], "launches_per_step": v[1]} for k, v in prof.items()}
    med = {k: statistics.median(v) for k, v in times.items()}
    ps = (med["lookup"] + med["table"]) / (1 << args.lookups_log) * 1e12
    dev.close()
    if rank != 0:
        return
    line = {
        "metric": "LogUp ps per lookup (fraction-tree build + level sumchecks, lookup and table trees)",
        "value": ps, "unit": "ps/lookup", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (Goldilocks Fp2)",
        "data": "synthetic (the reference benchmark's counter-generated keys, values and multiplicities)",
        "config": {"workload": f"2^{args.lookups_log} lookups into 2^{args.rows_log} rows, each tree its own proof",
                   "timing": "host wall clock per tree, median over steps, leaves generated on the device inside; "
                             "kernels from one more profiled step"},
        "lookup_tree_ms": med["lookup"] * 1e3, "table_tree_ms": med["table"] * 1e3,
        "reference_h100_ps_per_lookup": 297.0, "kernels": kernels,
    }
    print(json.dumps(line), flush=True)


CC_ID = bytes([0x5A]) * 32  # the commitment id of the reference benchmark's c_c run


def run_cc(args) -> None:
    """The reference benchmark's c_c measurement (crates/tessera-bench/examples/gpu_unit_costs.rs
    `cc`): rows of k = 2^cc_log_k values with P mask coefficients, generated on the device 32 rows
    at a time by the reference's counter generator (rows from counter 32·k·block, masks from
    2^62 + 32·P·block), encoded at rate 1/2 and absorbed into the 2k column chains (B = 32); the
    cost per committed element is (generate + encode + hash − generate) ÷ rows·k, medians over the
    timed runs, as the reference reports it. --impl refgpu runs the reference's own kernels the
    same way (oracle/refgpu.cpp)."""
    import ctypes

    import torch

    from tessera_gb300 import _native as N
    from tessera_gb300.device import Device

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    cuda = f"cuda:{local}"
    dev = Device(local)
    lgk, lgr, P_, B = args.cc_log_k, 1, args.cc_masks, ROW_BLOCK
    k, n = 1 << lgk, 1 << (lgk + lgr)
    blocks = args.cc_rows // B
    rows = torch.empty(B * k, dtype=torch.int64, device=cuda)
    masks = torch.empty(max(B * P_, 1), dtype=torch.int64, device=cuda)
    cw = torch.empty(B * n, dtype=torch.int64, device=cuda)
    chains = torch.empty(n * 32, dtype=torch.uint8, device=cuda)
    cid = (ctypes.c_uint8 * 32)(*CC_ID)
    torch.cuda.synchronize()
    v = ctypes.c_void_p
    stream = torch.cuda.ExternalStream(dev.stream_ptr(), device=cuda)

    def generate(b):
        N.call("tg_fill_counter", dev.handle, v(rows.data_ptr()), B * k, b * B * k, None)
        if P_:
            N.call("tg_fill_counter", dev.handle, v(masks.data_ptr()), B * P_, (1 << 62) + b * B * P_, None)

    def run(mode):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        if mode == 2:
            N.call("tg_column_init_dev", dev.handle, cid, n, v(chains.data_ptr()), None)
        for b in range(blocks):
            generate(b)
            if mode >= 1:
                N.call("tg_encode_rows_dev", dev.handle, lgk, lgr, P_, v(rows.data_ptr()), B,
                       v(masks.data_ptr()) if P_ else None, v(cw.data_ptr()), None)
            if mode == 2:
                N.call("tg_column_absorb_dev", dev.handle, v(chains.data_ptr()), n, v(cw.data_ptr()), B, B, None)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3

    def block0_chains():
        N.call("tg_column_init_dev", dev.handle, cid, n, v(chains.data_ptr()), None)
        generate(0)
        N.call("tg_encode_rows_dev", dev.handle, lgk, lgr, P_, v(rows.data_ptr()), B,
               v(masks.data_ptr()) if P_ else None, v(cw.data_ptr()), None)
        N.call("tg_column_absorb_dev", dev.handle, v(chains.data_ptr()), n, v(cw.data_ptr()), B, B, None)
        dev.sync()
        return chains.cpu().numpy().tobytes()

    elems = blocks * B * k
    impl = args.impl
    if impl == "refgpu":
        # the reference's kernels in their own module and stream; the library's chains of block 0
        # are computed first, on the same counter-generated inputs, to compare with theirs
        ours = block0_chains()
        del rows, masks, cw, chains
        torch.cuda.synchronize()
        dev.close()
        fatbin = ROOT / "oracle" / "_ref" / "commit.fatbin"
        lib_path = ROOT / "oracle" / "_build" / "librefgpu.so"
        if not fatbin.exists() or not lib_path.exists():
            if rank == 0:
                print(json.dumps({"impl": "refgpu", "unavailable": "the reference kernels were not compiled here "
                                  "(oracle/_ref/commit.fatbin needs the reference checkout; make -C oracle ref refgpu)"}))
            return
        from oracle import oracle as O

        lib = ctypes.CDLL(str(lib_path))
        lib.refgpu_last_error.restype = ctypes.c_char_p
        out = (ctypes.c_double * 3)()
        theirs = ctypes.create_string_buffer(n * 32)
        rc = lib.refgpu_cc(str(fatbin).encode(), ctypes.c_uint32(lgk), ctypes.c_uint32(args.cc_rows),
                           ctypes.c_uint32(P_), ctypes.c_int(args.warmup), ctypes.c_int(args.steps),
                           ctypes.c_int(O.threads_available()), out, theirs)
        if rc != 0:
            raise RuntimeError("reference kernels: " + lib.refgpu_last_error().decode())
        full, gen, enc = out[0], out[1], out[2]
        same = theirs.raw == ours
    else:
        for _ in range(args.warmup):
            run(2)
        full = statistics.median([run(2) for _ in range(args.steps)])
        gen = statistics.median([run(0) for _ in range(args.steps)])
        enc = statistics.median([run(1) for _ in range(args.steps)])
        same = None
        del rows, masks, cw, chains
        dev.close()
    if rank != 0:
        return
    ps = lambda t: t / elems * 1e12  # noqa: E731
    line = {
        "metric": "c_c: ps per committed element (encode at rate 1/2 with masks + BLAKE3 column chains)",
        "value": ps(full) - ps(gen), "unit": "ps/element", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u64 (Goldilocks)",
        "impl": impl,
        "data": "synthetic (the reference benchmark's counter generator on the device, 32 rows and their masks at a time)",
        "config": {"workload": f"{blocks * B} rows of k = 2^{lgk}, P = {P_} masks, rate 1/2, B = {B}",
                   "timing": "CUDA events over all blocks, median over steps"},
        "generate_encode_hash_ps": ps(full), "generate_ps": ps(gen), "encode_ps": ps(enc) - ps(gen),
        "hash_ps": ps(full) - ps(enc), "reference_h100_ps": 134.8,
    }
    if impl == "refgpu":
        line["kernels"] = ("the reference's crates/tessera-gpu/kernels/commit.cu (fill_counter, ntt_pass, encode_low, "
                           "column_init, column_step) compiled for sm_103 with its own flags, launched with the geometry "
                           "of crates/tessera-gpu/src/commit.rs; block 0 checked against the CPU oracle")
        line["block0_chains_equal_library"] = same
    print(json.dumps(line), flush=True)


def run_forest(args) -> None:
    """The reference benchmark's c_π measurement: one forest of 2^s product trees of 2^h prime-field
    leaves (the counter generator from 2^61, generated on the device before timing), its levels
    built bottom-up and its h degree-3 level sumchecks proven on a transcript (root challenges, γ,
    rounds, evals, ρ per level). The workspace is reused from one proof to the next, as the
    reference's is; the cost per leaf is the whole proof's time over 2^(s+h)."""
    import torch

    from tessera_gb300.device import Device
    from tessera_gb300.hash import Mode, SessionContext, Transcript
    from tessera_gb300.trees import Forest, LeafStage
    from tessera_gb300.workloads import fill_counter

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = Device(local)
    ctx = SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "test-small/1", bytes([0x65]) * 32, bytes([0x65]) * 16)
    s_, h_ = args.forest_trees_log, args.forest_leaves_log
    leaves = fill_counter(torch.empty(1 << (s_ + h_), dtype=torch.int64, device=f"cuda:{local}"), 1 << 61, dev)
    torch.cuda.synchronize()
    if args.impl == "refgpu":
        # the reference's own forest prover (oracle/refgpu.cpp over crates/tessera-gpu/kernels/trees.cu),
        # on its benchmark's transcript; the library proves the same forest on the same transcript
        # first, and the two final transcript states must agree (every message was absorbed)
        import ctypes

        bench_ctx = SessionContext("tessera-protocol/1", Mode.NON_INTERACTIVE, "bench/1", bytes([0x65]) * 32,
                                   bytes([0x13]) * 16)
        t = Transcript(bench_ctx)
        with LeafStage([Forest(s_, leaves, True)], dev) as st:
            st.prove(t)
        ours = (t.state, t.counter)
        del leaves
        torch.cuda.synchronize()
        dev.trim()
        dev.close()
        trees_fb, commit_fb = ROOT / "oracle" / "_ref" / "trees.fatbin", ROOT / "oracle" / "_ref" / "commit.fatbin"
        lib_path = ROOT / "oracle" / "_build" / "librefgpu.so"
        if not (trees_fb.exists() and commit_fb.exists() and lib_path.exists()):
            if rank == 0:
                print(json.dumps({"impl": "refgpu", "unavailable": "the reference kernels were not compiled here "
                                  "(oracle/_ref/{trees,commit}.fatbin need the reference checkout)"}))
            return
        lib = ctypes.CDLL(str(lib_path))
        lib.refgpu_last_error.restype = ctypes.c_char_p
        out = (ctypes.c_double * 1)()
        state = ctypes.create_string_buffer(32)
        counter = ctypes.c_uint64()
        rc = lib.refgpu_pi(str(trees_fb).encode(), str(commit_fb).encode(), ctypes.c_uint32(s_), ctypes.c_uint32(h_),
                           ctypes.c_int(args.warmup), ctypes.c_int(args.steps), out, state, ctypes.byref(counter))
        if rc != 0:
            raise RuntimeError("reference kernels: " + lib.refgpu_last_error().decode())
        if rank != 0:
            return
        print(json.dumps({
            "metric": "c_pi: ps per product-forest leaf (level build + level sumchecks on a transcript)",
            "value": out[0] / (1 << (s_ + h_)) * 1e12, "unit": "ps/leaf", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64 (Goldilocks; Fp2 after the first bind)", "impl": "refgpu",
            "data": "synthetic (counter-generated prime-field leaves on the device, as the reference benchmark)",
            "config": {"workload": f"one forest of 2^{s_} trees of 2^{h_} leaves",
                       "timing": "host wall clock per proof (leaves already on the device), median over steps"},
            "proof_ms": out[0] * 1e3,
            "kernels": "the reference's crates/tessera-gpu/kernels/trees.cu (tree_level, eq_table, level_sums_base, "
                       "bind_sums_base, bind_sums_ext, reduce_sums, bind_base, bind_ext) compiled for sm_103 with its "
                       "own flags, driven as crates/tessera-gpu/src/trees.rs prove_forest_in does",
            "final_transcript_equal_library": (state.raw, counter.value) == ours,
        }), flush=True)
        return

    def one():
        start = time.perf_counter()
        t = Transcript(ctx)
        with LeafStage([Forest(s_, leaves, True)], dev) as st:
            st.prove(t)
        torch.cuda.synchronize()
        return time.perf_counter() - start

    for _ in range(args.warmup):
        one()
    times = [one() for _ in range(args.steps)]  # timed without per-launch events
    dev.profile(True)  # one more proof, profiled, for the kernel breakdown
    one()
    dev.profile(False)
    prof = dev.profile_read()
    kernels = {k: {"ms_per_step": v[0], "launches_per_step": v[1]} for k, v in prof.items()}
    med = statistics.median(times)
    del leaves
    dev.close()
    if rank != 0:
        return
    line = {
        "metric": "c_pi: ps per product-forest leaf (level build + level sumchecks on a transcript)",
        "value": med / (1 << (s_ + h_)) * 1e12, "unit": "ps/leaf", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64 (Goldilocks; Fp2 after the first bind)",
        "data": "synthetic (counter-generated prime-field leaves on the device, as the reference benchmark)",
        "config": {"workload": f"one forest of 2^{s_} trees of 2^{h_} leaves",
                   "timing": "host wall clock per proof (leaves already on the device), median over steps; "
                             "kernels from one more profiled proof"},
        "proof_ms": med * 1e3, "reference_h100_ps_per_leaf": 84.6, "kernels": kernels,
    }
    print(json.dumps(line), flush=True)


SEED_SERVE = 0x00650005


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference", "refgpu"], default="gb300",
                    help="reference: the CPU port of the reference's algorithms; refgpu: the reference's own CUDA "
                         "kernels on this GPU (--workload cc, forest, logup)")
    ap.add_argument("--workload", choices=["large", "batched", "serve", "logup", "cc", "forest"], default="large",
                    help="large: the 256 x 2^20 commitment + 2^22 sumcheck headline; batched: batched vs plain; "
                         "serve: the proof server against one-at-a-time proofs")
    ap.add_argument("--requests", type=int, default=2000, help="serve: requests in the stream")
    ap.add_argument("--distinct", type=int, default=400,
                    help="serve: distinct input sets (request i proves input set i mod distinct, on its own transcript)")
    ap.add_argument("--lookups-log", type=int, default=30, help="logup: log2 of the lookups")
    ap.add_argument("--cc-log-k", type=int, default=22, help="cc: log2 of the row length")
    ap.add_argument("--forest-trees-log", type=int, default=16, help="forest: log2 of the trees")
    ap.add_argument("--forest-leaves-log", type=int, default=14, help="forest: log2 of each tree's leaves")
    ap.add_argument("--cc-masks", type=int, default=200, help="cc: mask coefficients per row")
    ap.add_argument("--cc-rows", type=int, default=4096, help="cc: rows committed per run")
    ap.add_argument("--rows-log", type=int, default=24, help="logup: log2 of the table rows")
    ap.add_argument("--rate", type=float, default=20.0, help="serve: mean Poisson arrivals per second")
    ap.add_argument("--slots", type=int, default=8, help="serve: requests in flight at most")
    ap.add_argument("--queries", type=int, default=32,
                    help="serve: column queries each request answers from its resident commitment after the proof")
    ap.add_argument("--serve-budget-gib", type=int, default=64, help="serve: HBM budget for admitted requests")
    ap.add_argument("--cpu-polys", type=int, default=32, help="rows encoded per run in the CPU baseline's sample")
    ap.add_argument("--ref-polys", type=int, default=32, help="rows encoded per run in the reference arm's sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--lde-group-mib", type=int, default=0, help="encoder scratch per group of rows (0: the library default)")
    ap.add_argument("--polys", type=int, default=NPOLYS,
                    help="rows committed per step (a smaller case for profiler captures; the headline uses 256)")
    args = ap.parse_args()
    if args.polys != NPOLYS:
        global COMMITTED, UNITS
        COMMITTED = args.polys << LOG_K
        UNITS = COMMITTED + SUMCHECKED
        CONFIG["polys"] = args.polys
        CONFIG["workload"] = CONFIG["workload"].replace("commit 256", f"commit {args.polys}")
    if args.impl == "refgpu" and args.workload not in ("cc", "forest", "logup"):
        print(json.dumps({"impl": "refgpu", "unavailable": "the reference's own kernels are driven for --workload cc, forest and logup"}))
    elif args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "serve":
        run_serve(args)
    elif args.workload == "logup":
        run_logup(args)
    elif args.workload == "cc":
        run_cc(args)
    elif args.workload == "forest":
        run_forest(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
