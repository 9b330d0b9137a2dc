"""Benchmark of the regular-force hot path (gpunb_send_ + gpunb_regf_).

Workload (default): Plummer N = 65536 in Henon units, Kroupa masses, RS for a
mean of 100 neighbours, nbmax 512.  One step = the five regular blocks of a
block-time-step hierarchy, ni in {1, 32, 1024, 16384, 65536}; each block is a
full j-set upload (send) plus one regf call, as the integrator does it
(src/Main/intgrt.F:912-944).  Metric: pairs (ni * N summed over the blocks)
per second, in Gpairs/s.

  value  device-resident inputs (j- and i-arrays already in HBM), timed with
         CUDA events on the stream the library launches on;
  e2e    the same step through the C ABI with host arrays (gpunb_send_,
         gpunb_regf_), host<->device copies included, wall clock;
  fp64   the plain FP64 kernel on the same step (the metric's "vs FP64").
  double_float  the same step in double-float arithmetic on the FP32 pipe.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

BLOCKS = [1, 32, 1024, 16384, 65536]
N = 65536
NB_TARGET = 100.0
NNBMAX = 512
LMAX = NNBMAX + 1
FLOPS_PER_PAIR = 60          # the reference's convention (gpunb.velocity.cu:894)
RESORT_EVERY = 8             # j-set re-ordered on every 8th send (the library's default)
METRIC = "regular force+jerk+NB Gpairs/s on 1 GB300: split-FP32 vs FP64 at rel.err<=1e-6"
WORKLOAD = "plummer65536_kroupa_blocks_1_32_1024_16384_65536"


def _jsonable(o):
    """numpy scalars and arrays in the bench line as plain JSON values"""
    if isinstance(o, np.generic):
        return o.item()
    if isinstance(o, np.ndarray):
        return o.tolist()
    raise TypeError(f"not JSON serialisable: {type(o).__name__}")


def config(ws: int = 1) -> dict:
    """The workload's config, identical in both arms of the bench."""
    return {"workload": WORKLOAD, "N": N, "blocks": BLOCKS, "nb_target": NB_TARGET,
            "nnbmax": NNBMAX, "l2": "flushed (256 MB write) between timed steps",
            "parallelism": f"replicas x{ws}"}


def make_inputs(seed: int = 2):
    from nbody6ppgpu_gb300 import ics
    c = ics.plummer(N, seed=seed, masses="kroupa", nb_target=NB_TARGET)
    acts = {ni: ics.active_set(N, ni, seed=ni) for ni in BLOCKS}
    return c, acts


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = Path("/tmp") / f"bench_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        # start timing only once the sampler is running (first line written)
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            if self.path.exists() and self.path.stat().st_size > 0:
                break
            time.sleep(0.01)

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
                power.append(float(f[3]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(name)
        self.path.unlink(missing_ok=True)
        load = [s for s in sm if smax and s > 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


def gpu_info():
    import torch
    p = torch.cuda.get_device_properties(0)
    return p.name, p.multi_processor_count


def fp32_peak_tflops(n_sm: int, mhz: float) -> float:
    # 128 FP32 lanes per SM, 2 flops per FMA
    return n_sm * 128 * 2 * mhz * 1e6 / 1e12


def fp64_peak_tflops(n_sm: int, mhz: float) -> float:
    # 2 FP64 FMAs per SM per cycle on GB300 (ncu: dfma peak 2 per cycle per SM)
    return n_sm * 2 * 2 * mhz * 1e6 / 1e12


def hbm_gbs() -> float:
    """Measured copy bandwidth of the GB300s (MEASURED_PEAKS.json), else 6800."""
    try:
        return float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        return 6800.0


# j-tile bytes per body (TILE_BYTES / JT of the library: 12 fields + metadata, 128
# bodies), read once per i-tile pass; i-tile sizes of the launch shapes
TILE_BYTES_PER_BODY = 6704 / 128


def read_traffic():
    """DRAM bytes per launch of the pair kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "regf_ds_kernel_plummer65536.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


# --------------------------------------------------------------------------
def oracle_parity(name, m, x, v, h2, dtr, act, got, lmax, nnbmax, rows=512):
    """Sampled rows of a split-precision block against the FP64 oracle:
    the named bound of oracle.parity_errors (force and jerk against
    max(|Q|, sum|q|/8), potential relative) next to the plain relative
    maxima and 99th percentiles."""
    from oracle import oracle as O
    acc, jrk, pot = got
    samp = np.linspace(0, len(act) - 1, min(rows, len(act))).astype(int)
    a = act[samp]
    oa, oj, op, lst, aa, ja = O.regf_fp64(m, x, v, h2[a], dtr[a], x[a], v[a], lmax, nnbmax,
                                          with_abs=True)
    ok = lst[:, 0] >= 0
    e = O.parity_errors(acc[samp][ok], jrk[samp][ok], pot[samp][ok], oa[ok], oj[ok], op[ok],
                        aa[ok], ja[ok])
    e["block"] = name
    e["rows_sampled"] = int(ok.sum())
    return e


def cpu_side_checks(c, irr_check=None, pot_result=None):
    """The CPU-baseline leg's work for the side legs: the irregular force of
    the FP64 oracle (timed, and the GPU block checked against it) and the
    potential of the FP32 port (timed) and of the FP64 oracle (check)."""
    from oracle import oracle as O
    out = {}
    if irr_check is not None:
        st = irr_check["state"]
        act = st[-1]
        lists = st[6]
        O.irr_fp64(*st)
        t = time.perf_counter()
        oa, oj, on = O.irr_fp64(*st)
        dt = time.perf_counter() - t
        ok = np.linalg.norm(oa, axis=1) > 0
        a, j, nid = irr_check["gpu"]["fp64"]
        ea = np.linalg.norm(a[ok] - oa[ok], axis=1) / np.linalg.norm(oa[ok], axis=1)
        sa, sj = O.irr_abs_sums(*st)
        a, j, nid_d = irr_check["gpu"]["double_float"]
        ed = max(float((np.linalg.norm(a[ok] - oa[ok], axis=1) / np.linalg.norm(oa[ok], axis=1)).max()),
                 float((np.linalg.norm(j[ok] - oj[ok], axis=1) / np.linalg.norm(oj[ok], axis=1)).max()))
        a, j, nid_s = irr_check["gpu"]["split"]
        ones = np.ones(len(act))
        pe = O.parity_errors(a[ok], j[ok], ones[ok], oa[ok], oj[ok], ones[ok], sa[ok], sj[ok])
        pe.pop("pot")
        out["irregular"] = {"kind": "FP64 oracle (oracle/irr_fp64.c)", "cores": O.num_threads(),
                            "ni": int(len(act)),
                            "gpairs_s": int(lists[act, 0].sum()) / dt / 1e9,
                            "gpu_fp64_max_rel_err_vs_fp64_oracle": float(ea.max()),
                            "gpu_fp64_nnbid_identical": bool(np.array_equal(nid, on)),
                            "gpu_double_float_max_rel_err_vs_fp64_oracle": ed,
                            "gpu_double_float_nnbid_identical": bool(np.array_equal(nid_d, on)),
                            "gpu_split_parity_vs_fp64_oracle": pe,
                            "gpu_split_nnbid_differing": int(np.sum(nid_s != on))}
    if pot_result is not None:
        n = c.n
        t = time.perf_counter()
        O.Port.pot(c.m, c.x)
        dt = time.perf_counter() - t
        ref = O.pot_fp64(c.m, c.x, 1, 2048)
        out["potential"] = {"kind": "port (FP32 restatement of src/Main/pot.avx.cpp)",
                            "cores": O.num_threads(), "gpairs_s": n * n / dt / 1e9,
                            "gpu_max_rel_err_vs_fp64_oracle":
                                float(np.max(np.abs(pot_result[:2048] - ref) / ref))}
    return out


def cpu_baseline(c, acts, sample_s: float = 10.0):
    """The portable FP32 restatement of the reference CPU path (OpenMP, all
    host cores) on whole steps of the same workload, as many as fit in
    about sample_s (at least one)."""
    from oracle import oracle as O
    port = O.Port()
    h2 = c.h2()
    pairs = 0
    steps = 0
    t0 = time.perf_counter()
    while True:
        for ni in BLOCKS:
            a = acts[ni]
            port.send(c.m, c.x, c.v)
            port.regf(h2[a], c.dtr[a], c.x[a], c.v[a], LMAX, NNBMAX)
            pairs += ni * N
        steps += 1
        if time.perf_counter() - t0 > sample_s or steps >= 20:
            break
    dt = time.perf_counter() - t0
    return {"value": pairs / dt / 1e9, "unit": "Gpairs/s", "cores": O.num_threads(),
            "kind": "port",
            "sample": f"{steps} full step(s) of the workload ({pairs:.3e} pairs) with the FP32 "
                      f"restatement of src/Main/reg.avx.cpp (x86 AVX source does not build on "
                      f"this aarch64 host)"}, pairs / dt


def run_reference(args, ws, rank):
    """--impl reference: the reference's CPU path (portable restatement) timed
    on the host cores; each step is one full step of the workload."""
    if rank != 0:
        return 0
    c, acts = make_inputs()
    from oracle import oracle as O
    port = O.Port()
    h2 = c.h2()

    def step():
        for ni in BLOCKS:
            a = acts[ni]
            port.send(c.m, c.x, c.v)
            port.regf(h2[a], c.dtr[a], c.x[a], c.v[a], LMAX, NNBMAX)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    pairs = N * sum(BLOCKS) * args.steps
    v = pairs / dt / 1e9
    line = {"metric": METRIC, "value": v, "unit": "Gpairs/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Plummer/Kroupa)",
            "config": config(args.gpus),
            "impl_detail": {"host_threads": O.num_threads(),
                            "code": "FP32 restatement of src/Main/reg.avx.cpp (OpenMP)"},
            "cpu_baseline": {"value": v, "unit": "Gpairs/s", "cores": O.num_threads(),
                             "kind": "port",
                             "sample": "every step = the full workload step on the host cores "
                                       "(FP32 restatement of src/Main/reg.avx.cpp; the x86 AVX "
                                       "source does not build on the aarch64 host)"},
            "e2e": {"value": v, "unit": "Gpairs/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line, default=_jsonable), flush=True)
    return 0


# --------------------------------------------------------------------------
def batched_leg(lib, dev, stream, steps: int, warmup: int):
    """256 independent Plummer clusters (N log-uniform in
    [512, 16384], active fraction log-uniform in [2^-10, 1], neighbour target
    U[50, 150]), every step one batched send + regf in a single persistent
    launch replayed from a CUDA graph, against one send + regf per cluster."""
    import torch
    from nbody6ppgpu_gb300 import workloads
    from nbody6ppgpu_gb300.batch import DeviceBatch
    sets, active, h2, dtr, _ = workloads.clusters256()
    nnbmax = 512
    b = DeviceBatch(sets, active, nnbmax, device=dev.index, stream=stream)
    b.set_radii(h2, dtr)
    pairs = int(sum(len(s[0]) * len(a) for s, a in zip(sets, active)))
    lib.gpunb_set_graphs(1)

    def step():
        b.send()
        b.regf()

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    batched_ms = e0.elapsed_time(e1) / steps
    lib.gpunb_set_graphs(0)
    variant, items = b.last_plan()
    # one gpunb_send_device + gpunb_regf_device per cluster, same buffers
    joff = np.concatenate([[0], np.cumsum(b.nj)])
    ioff = np.concatenate([[0], np.cumsum(b.ni)])
    scratch_off = torch.empty(int(b.ni.max()) + 1, dtype=torch.int32, device=dev)
    scratch_lst = torch.empty(int(b.ni.max()) * nnbmax, dtype=torch.int32, device=dev)
    sp = stream.cuda_stream

    def seq_pass():
        for c in range(b.ncl):
            j0, i0, ni = int(joff[c]), int(ioff[c]), int(b.ni[c])
            rc = lib.gpunb_send_device(int(b.nj[c]), b.m.data_ptr() + 8 * j0,
                                       b.x.data_ptr() + 24 * j0, b.v.data_ptr() + 24 * j0, sp)
            assert rc == 0
            rc = lib.gpunb_regf_device(ni, b.h2.data_ptr() + 8 * i0, b.dtr.data_ptr() + 8 * i0,
                                       b.xi.data_ptr() + 24 * i0, b.vi.data_ptr() + 24 * i0,
                                       b.acc.data_ptr() + 24 * i0, b.jrk.data_ptr() + 24 * i0,
                                       b.pot.data_ptr() + 8 * i0, b.nnb.data_ptr() + 4 * i0,
                                       scratch_off.data_ptr(), scratch_lst.data_ptr(),
                                       ni * nnbmax, nnbmax, 0, sp)
            assert rc == 0

    seq_pass()
    torch.cuda.synchronize()
    e0.record(stream)
    seq_pass()
    e1.record(stream)
    torch.cuda.synchronize()
    seq_ms = e0.elapsed_time(e1)
    return {"workload": "256 Plummer clusters, N log-uniform [512,16384], Kroupa, active "
                        "fraction log-uniform [2^-10,1], target U[50,150], nbmax 512",
            "bodies": int(b.nj.sum()), "active": int(b.ni.sum()), "pairs_per_step": pairs,
            "value": pairs / (batched_ms * 1e-3) / 1e9, "unit": "Gpairs/s",
            "ms_per_step": batched_ms, "graph": True, "variant": variant, "work_items": items,
            "sequential_value": pairs / (seq_ms * 1e-3) / 1e9, "sequential_ms": seq_ms,
            "speedup_over_sequential": seq_ms / batched_ms}


KING_BLOCKS = [1024, 16384, 262144, 1 << 20]
KING_NNBMAX = 1024


def king1m_leg(lib, dev, stream, n_sm: int, peak_mhz: float, steps: int = 2, warmup: int = 2):
    """The King 2^20 configuration as a full regular step: King W0 = 6,
    N = 2^20, Kroupa masses with 10% binaries as c.m. bodies, RS for a mean of
    100 neighbours, nbmax 1024; one step = send + regf for each block
    ni in {1024, 16384, 262144, N} (1.39e12 pairs).
      step      device-resident (gpunb_send_device + gpunb_regf_device on the
                timed stream, calls replayed as CUDA graphs), CUDA events per
                step, clocks sampled during the timed steps;
      e2e       the same step through gpunb_send_ / gpunb_regf_ with host
                arrays (copies and LISTGP rows included), wall clock;
      blocks    pair-kernel time of each block (library CUDA events) and its
                fraction of the FP32 peak: the roofline at ni = N;
      fp64      the FP64 kernel on the ni = 16384 block.
    Returns the line entry and what the oracle leg needs (the split results
    of the 16384 block for the parity check, the 1024 block for the CPU
    port's timing)."""
    import torch
    from nbody6ppgpu_gb300 import ics
    from nbody6ppgpu_gb300.gpunb import GpuNb
    t0 = time.perf_counter()
    k = ics.king(1 << 20, seed=4, nb_target=100.0)
    t_ics = time.perf_counter() - t0
    n = k.n
    h2 = k.h2()
    peak = fp32_peak_tflops(n_sm, peak_mhz)
    acts = {ni: ics.active_set(n, ni, seed=ni) for ni in KING_BLOCKS}
    pairs = n * sum(KING_BLOCKS)
    sp = stream.cuda_stream

    def T(a, dt=torch.float64):
        return torch.as_tensor(np.ascontiguousarray(a)).to(dev, dtype=dt)

    jm, jx, jv = T(k.m), T(k.x), T(k.v)
    blk = {}
    for ni in KING_BLOCKS:
        a = acts[ni]
        blk[ni] = dict(h2=T(h2[a]), dtr=T(k.dtr[a]), x=T(k.x[a]), v=T(k.v[a]),
                       acc=torch.empty((ni, 3), dtype=torch.float64, device=dev),
                       jrk=torch.empty((ni, 3), dtype=torch.float64, device=dev),
                       pot=torch.empty(ni, dtype=torch.float64, device=dev),
                       nnb=torch.empty(ni, dtype=torch.int32, device=dev),
                       off=torch.empty(ni + 1, dtype=torch.int32, device=dev),
                       lst=torch.empty(ni * KING_NNBMAX, dtype=torch.int32, device=dev))

    def dev_step():
        for ni in KING_BLOCKS:
            b = blk[ni]
            assert lib.gpunb_send_device(n, jm.data_ptr(), jx.data_ptr(), jv.data_ptr(), sp) == 0
            assert lib.gpunb_regf_device(ni, b["h2"].data_ptr(), b["dtr"].data_ptr(),
                                         b["x"].data_ptr(), b["v"].data_ptr(),
                                         b["acc"].data_ptr(), b["jrk"].data_ptr(),
                                         b["pot"].data_ptr(), b["nnb"].data_ptr(),
                                         b["off"].data_ptr(), b["lst"].data_ptr(),
                                         ni * KING_NNBMAX, KING_NNBMAX, 0, sp) == 0

    out = {"workload": "King W0=6, N=2^20, Kroupa, 10% binaries as c.m. bodies, target 100, "
                       "nbmax 1024; one step = send + regf at ni in {1024, 16384, 262144, N}",
           "setup_s": t_ics, "pairs_per_step": pairs}
    # launch shapes: the library's measured heuristic (its sweeps were taken on
    # this model); tuning ni = 2^20 on first sight would time ~100 passes of a
    # one-second kernel
    autotune_prev = lib.gpunb_set_autotune(0)
    with GpuNb(n) as nb:
        nb.set_precision("split")
        # device-resident steps, graphs on
        lib.gpunb_set_graphs(1)
        for _ in range(warmup):
            dev_step()
        torch.cuda.synchronize()
        clocks = Clocks(dev.index)
        clocks.start()
        evs = []
        for _ in range(steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dev_step()
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        clk = clocks.stop()
        lib.gpunb_set_graphs(0)
        step_ms = float(np.mean([a.elapsed_time(b) for a, b in evs]))
        got16 = (blk[16384]["acc"].cpu().numpy(), blk[16384]["jrk"].cpu().numpy(),
                 blk[16384]["pot"].cpu().numpy())
        nnb = {ni: blk[ni]["nnb"].cpu().numpy() for ni in KING_BLOCKS}
        # per-block pair-kernel times: one step without graphs, library events
        nb.set_timing(True)
        dev_step()
        torch.cuda.synchronize()
        kt = [float(t) for t in nb.kernel_times()]
        nb.set_timing(False)
        blocks = {}
        for q, ni in enumerate(KING_BLOCKS):
            gp = ni * n / (kt[q] * 1e-3) / 1e9
            blocks[str(ni)] = {"kernel_ms": float(kt[q]), "gpairs_s": gp,
                               "frac_fp32": gp * 1e9 * FLOPS_PER_PAIR / 1e12 / peak,
                               "overflows": int((nnb[ni] < 0).sum()),
                               "mean_neighbours": float(np.maximum(nnb[ni], 0).mean())}
        # FP64 kernel on the 16384 block
        nb.set_precision("fp64")
        nb.set_timing(True)
        b = blk[16384]
        assert lib.gpunb_send_device(n, jm.data_ptr(), jx.data_ptr(), jv.data_ptr(), sp) == 0
        assert lib.gpunb_regf_device(16384, b["h2"].data_ptr(), b["dtr"].data_ptr(),
                                     b["x"].data_ptr(), b["v"].data_ptr(), b["acc"].data_ptr(),
                                     b["jrk"].data_ptr(), b["pot"].data_ptr(),
                                     b["nnb"].data_ptr(), b["off"].data_ptr(),
                                     b["lst"].data_ptr(), 16384 * KING_NNBMAX, KING_NNBMAX, 0,
                                     sp) == 0
        torch.cuda.synchronize()
        fp64_ms = float(nb.kernel_times()[-1])
        nb.set_timing(False)
        a64 = (b["acc"].cpu().numpy(), b["jrk"].cpu().numpy(), b["pot"].cpu().numpy())
        nb.set_precision("split")
        del blk
        torch.cuda.empty_cache()
        # end to end through the host ABI, graphs on
        hin = {ni: (h2[acts[ni]].copy(), k.dtr[acts[ni]].copy(), k.x[acts[ni]].copy(),
                    k.v[acts[ni]].copy()) for ni in KING_BLOCKS}
        outs = {}

        def host_step():
            for ni in KING_BLOCKS:
                nb.send(k.m, k.x, k.v)
                outs[ni] = nb.regf(*hin[ni], KING_NNBMAX + 1, KING_NNBMAX, out=outs.get(ni))

        # the first steps capture the graphs and touch the caller's host arrays
        # for the first time (4.3 GB of LISTGP rows at ni = N): warm up fully
        lib.gpunb_set_graphs(1)
        for _ in range(max(2, warmup)):
            host_step()
        e2e_steps = max(3, steps)
        t = time.perf_counter()
        for _ in range(e2e_steps):
            host_step()
        e2e_s = (time.perf_counter() - t) / e2e_steps
        lib.gpunb_set_graphs(0)
    lib.gpunb_set_autotune(autotune_prev)
    h2d = sum(56 * n + 64 * ni for ni in KING_BLOCKS)
    d2h = sum(60 * ni + 4 * int(np.maximum(outs[ni].list[:, 0], 0).sum()) for ni in KING_BLOCKS)
    a, j, p = got16
    ea = np.linalg.norm(a - a64[0], axis=1) / np.linalg.norm(a64[0], axis=1)
    ej = np.linalg.norm(j - a64[1], axis=1) / np.linalg.norm(a64[1], axis=1)
    ep = np.abs(p - a64[2]) / np.abs(a64[2])
    fp64_gp = 16384 * n / (fp64_ms * 1e-3) / 1e9
    big = blocks[str(n)]
    achieved = big["gpairs_s"] * FLOPS_PER_PAIR / 1e3
    out.update({
        "value": pairs / (step_ms * 1e-3) / 1e9, "unit": "Gpairs/s", "step_ms": step_ms,
        "steps": steps, "warmup": warmup, "clocks": clk,
        "e2e": {"value": pairs / e2e_s / 1e9, "unit": "Gpairs/s", "step_s": e2e_s,
                "steps": e2e_steps, "warmup": max(2, warmup),
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "blocks": blocks,
        "roofline": {"bound": "fp32", "kernel": "regf_ds_kernel (ni = N block)",
                     "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "flops_per_pair": FLOPS_PER_PAIR},
        "fp64_ni16384": {"kernel_ms": fp64_ms, "gpairs_s": fp64_gp},
        "speedup_split_over_fp64_kernel_ni16384": blocks["16384"]["gpairs_s"] / fp64_gp,
        "speedup_split_ni_N_over_fp64_kernel": big["gpairs_s"] / fp64_gp,
        "rel_err_vs_fp64_kernel_ni16384": {
            "acc_p99": float(np.percentile(ea, 99)), "acc_max": float(ea.max()),
            "jrk_p99": float(np.percentile(ej, 99)), "jrk_max": float(ej.max()),
            "pot_max": float(ep.max())}})
    check = ("King N=2^20 ni=16384", k.m, k.x, k.v, h2, k.dtr, acts[16384], got16,
             KING_NNBMAX + 1, KING_NNBMAX)
    cpu_block = (k, h2, acts[1024])
    return out, check, cpu_block


def king_cpu_block(k, h2, act):
    """The FP32 port on the King 2^20 set: one block of 1024 active bodies
    against all N (1.07e9 pairs) on the host cores."""
    from oracle import oracle as O
    port = O.Port()
    port.send(k.m, k.x, k.v)
    t = time.perf_counter()
    port.regf(h2[act], k.dtr[act], k.x[act], k.v[act], KING_NNBMAX + 1, KING_NNBMAX)
    dt = time.perf_counter() - t
    return {"value": len(act) * k.n / dt / 1e9, "unit": "Gpairs/s", "cores": O.num_threads(),
            "kind": "port", "sample": f"one block of {len(act)} active bodies against all "
                                      f"{k.n} (FP32 restatement of src/Main/reg.avx.cpp)"}


def irregular_leg(c, h2, lists_src, dev=None):
    """Irregular (neighbour) force through the irr_simd_* ABI (the drop-in
    for src/Main/irr.avx.cpp): the bench's Plummer N = 65536 with the
    neighbour lists of its ni = 65536 regular block (the particle itself
    removed), predictor state from that block's regular force, blocks of
    1024, 16384 and 65536 particles at a common time, in split precision
    (the default) and in FP64.  Host-ABI calls are timed on the wall clock;
    the device-resident form (irr_firr_device) with CUDA events on its
    stream.  Unit: listed pairs."""
    import ctypes as C

    import torch

    from nbody6ppgpu_gb300.gpunb import load
    from nbody6ppgpu_gb300.irr import IrrSimd
    n = c.n
    lmax = lists_src.shape[1]
    lists = np.zeros_like(lists_src)
    for i in range(n):
        cnt = max(int(lists_src[i, 0]), 0)
        ids = lists_src[i, 1:1 + cnt]
        ids = ids[ids != i]
        lists[i, 0] = len(ids)
        lists[i, 1:1 + len(ids)] = ids
    rng = np.random.default_rng(7)
    f = rng.normal(0.0, 0.5, (n, 3))
    fdot = rng.normal(0.0, 0.5, (n, 3))
    ti = 1.0
    t0 = ti - rng.uniform(0.0, 2e-3, n)
    blocks = {ni: rng.permutation(n)[:ni] for ni in (1024, 16384, n)}
    out = {"workload": "Plummer N=65536 (the bench cluster), lists of its regular block",
           "precision": "double-float on the FP32 pipe (the default), fp64 "
                        "(irr_set_precision(1)) and split FP32 (irr_set_precision(0): "
                        "double-single positions); an FP64 prediction in every mode",
           "host_abi": {"double_float": {}, "split": {}, "fp64": {}},
           "device": {"double_float": {}, "split": {}, "fp64": {}}}
    with IrrSimd(n, lmax) as irr:
        irr.set_jp(c.x, c.v, f, fdot, c.m, t0)
        irr.set_lists(lists)
        for prec, key in ((2, "double_float"), (0, "split"), (1, "fp64")):
            irr.set_precision(prec)
            for ni, act in blocks.items():
                pairs = int(lists[act, 0].sum())
                # the caller's result arrays persist between calls (as Fortran's)
                res = (np.zeros((ni, 3)), np.zeros((ni, 3)), np.zeros(ni, dtype=np.int32))
                irr.firr(ti, act, out=res)
                best = 1e9
                for _ in range(5):
                    t = time.perf_counter()
                    irr.firr(ti, act, out=res)
                    best = min(best, time.perf_counter() - t)
                out["host_abi"][key][str(ni)] = {"pairs": pairs, "ms": best * 1e3,
                                                 "gpairs_s": pairs / best / 1e9}
        irr.set_precision(2)
        # predict-and-send from the stored state vs gpunb_send_ of host arrays
        from nbody6ppgpu_gb300.gpunb import GpuNb
        from nbody6ppgpu_gb300.irr import send_predicted
        with GpuNb(n) as nb:
            tp, ts = [], []
            for _ in range(6):
                t = time.perf_counter()
                xp, vp = send_predicted(ti, c.m)
                tp.append(time.perf_counter() - t)
                t = time.perf_counter()
                nb.send(c.m, xp, vp)
                ts.append(time.perf_counter() - t)
        out["predict_send_ms"] = 1e3 * min(tp[1:])
        out["send_host_arrays_ms"] = 1e3 * min(ts[1:])
    # the device-resident form, kernels timed with CUDA events on their stream
    dev = dev or torch.device("cuda", 0)
    rec = np.zeros((n, 16))
    rec[:, 0:3] = c.x; rec[:, 3] = c.m; rec[:, 4:7] = c.v; rec[:, 7] = t0
    rec[:, 8:11] = f; rec[:, 12:15] = fdot
    R = torch.tensor(rec, device=dev)
    L = torch.tensor(lists, device=dev)
    lib = load()
    fn = lib.irr_firr_device
    fn.argtypes = [C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_int, C.c_void_p,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    st = torch.cuda.Stream(dev)
    for prec, key in ((2, "double_float"), (0, "split"), (1, "fp64")):
        lib.irr_set_precision(prec)
        for ni, act in blocks.items():
            A = torch.tensor(act.astype(np.int32), device=dev)
            acc = torch.empty(ni, 3, dtype=torch.float64, device=dev)
            jrk = torch.empty_like(acc)
            nid = torch.empty(ni, dtype=torch.int32, device=dev)
            args = (n, R.data_ptr(), lmax, L.data_ptr(), ti, ni, A.data_ptr(), acc.data_ptr(),
                    jrk.data_ptr(), nid.data_ptr(), st.cuda_stream)
            torch.cuda.synchronize()
            for _ in range(3):
                assert fn(*args) == 0
            reps = 20
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(st):
                e0.record(st)
                for _ in range(reps):
                    fn(*args)
                e1.record(st)
            e1.synchronize()
            ms = e0.elapsed_time(e1) / reps
            pairs = int(lists[act, 0].sum())
            out["device"][key][str(ni)] = {"ms": ms, "gpairs_s": pairs / ms / 1e6}
    lib.irr_set_precision(2)
    s16, f16 = out["device"]["split"][str(n)], out["device"]["fp64"][str(n)]
    d16 = out["device"]["double_float"][str(n)]
    out["device"]["split_over_fp64_ni65536"] = f16["ms"] / s16["ms"]
    out["device"]["double_float_over_fp64_ni65536"] = f16["ms"] / d16["ms"]
    # a block of 16384 for the CPU-baseline leg (timing and the FP64 checks)
    act = blocks[16384]
    res = {}
    with IrrSimd(n, lmax) as irr:
        irr.set_jp(c.x, c.v, f, fdot, c.m, t0)
        irr.set_lists(lists)
        for prec, key in ((2, "double_float"), (0, "split"), (1, "fp64")):
            irr.set_precision(prec)
            res[key] = irr.firr(ti, act)
        irr.set_precision(2)
    check = {"state": (c.x, c.v, f, fdot, c.m, t0, lists, ti, act), "gpu": res}
    return out, check


def potential_leg(c):
    """gpupot_ (the energy check's potential, gpupot.gpu.cu:61-127) over all
    bodies of the bench cluster, host ABI.  Returns the line entry and the
    result (checked against the FP64 oracle in the CPU-baseline leg)."""
    from nbody6ppgpu_gb300.gpunb import gpupot
    n = c.n
    gpupot(c.m, c.x)
    best = 1e9
    for _ in range(5):
        t = time.perf_counter()
        p = gpupot(c.m, c.x)
        best = min(best, time.perf_counter() - t)
    out = {"workload": "Plummer N=65536 (the bench cluster), all bodies, host ABI",
           "ms": best * 1e3, "gpairs_s": n * n / best / 1e9}
    return out, p


def rs_predictor_leg(dev):
    """Inference of the neighbour-radius MLP for 2^20 particles (one forward
    kernel): 2^20 x (8*64 + 64*64 + 64) multiply-adds."""
    import torch
    from nbody6ppgpu_gb300.rsmlp import RSMLP
    m = RSMLP(seed=0, device=dev.index)
    B = 1 << 20
    X = torch.randn(B, 8, device=dev)
    y = torch.empty(B, device=dev)
    sp = m.stream.cuda_stream
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    for _ in range(3):
        assert m.lib.gpunb_rsmlp_forward(B, X.data_ptr(), m.wq.data_ptr(), m.master.data_ptr(),
                                         y.data_ptr(), sp) == 0
    reps = 10
    e0.record(m.stream)
    for _ in range(reps):
        m.lib.gpunb_rsmlp_forward(B, X.data_ptr(), m.wq.data_ptr(), m.master.data_ptr(),
                                  y.data_ptr(), sp)
    e1.record(m.stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    macs = B * (8 * 64 + 64 * 64 + 64)
    return {"particles": B, "forward_ms": ms, "gmacs_per_s": macs / (ms * 1e-3) / 1e9,
            "kernel": "rsmlp_forward_tc_kernel (mma.sync BF16 tiles, FP32 accumulation)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=64)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-large", action="store_true", help="skip the N = 2^20 King leg")
    ap.add_argument("--no-irregular", action="store_true", help="skip the irregular-force leg")
    ap.add_argument("--tune-save", default=None,
                    help="save the autotuner's cache here at the end (GPUNB_TUNE_CACHE=path "
                         "loads it in a later run, which then tunes nothing)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)

    import torch
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    from nbody6ppgpu_gb300.gpunb import GpuNb, load
    lib = load()
    # launch shapes from the autotuner: each block's (N, ni) bucket is tuned
    # on its first call (a warm-up call, untimed) and cached
    lib.gpunb_set_autotune(1)
    c, acts = make_inputs()
    h2 = c.h2()
    dev = torch.device("cuda", local)
    # a dedicated stream: the library and the timing events share it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    assert sp != 0

    def T(a, dt=torch.float64):
        return torch.as_tensor(np.ascontiguousarray(a)).to(dev, dtype=dt)

    jm, jx, jv = T(c.m), T(c.x), T(c.v)
    blk = {}
    for ni in BLOCKS:
        a = acts[ni]
        blk[ni] = dict(h2=T(h2[a]), dtr=T(c.dtr[a]), x=T(c.x[a]), v=T(c.v[a]),
                       acc=torch.empty((ni, 3), dtype=torch.float64, device=dev),
                       jrk=torch.empty((ni, 3), dtype=torch.float64, device=dev),
                       pot=torch.empty(ni, dtype=torch.float64, device=dev),
                       nnb=torch.empty(ni, dtype=torch.int32, device=dev),
                       off=torch.empty(ni + 1, dtype=torch.int32, device=dev),
                       lst=torch.empty(ni * NNBMAX, dtype=torch.int32, device=dev))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)   # > L2 (126 MB)

    nb = GpuNb(N)

    launch_plan = {}

    def dev_step():
        for ni in BLOCKS:
            b = blk[ni]
            rc = lib.gpunb_send_device(N, jm.data_ptr(), jx.data_ptr(), jv.data_ptr(), sp)
            assert rc == 0, rc
            rc = lib.gpunb_regf_device(ni, b["h2"].data_ptr(), b["dtr"].data_ptr(),
                                       b["x"].data_ptr(), b["v"].data_ptr(),
                                       b["acc"].data_ptr(), b["jrk"].data_ptr(),
                                       b["pot"].data_ptr(), b["nnb"].data_ptr(),
                                       b["off"].data_ptr(), b["lst"].data_ptr(),
                                       ni * NNBMAX, NNBMAX, 0, sp)
            assert rc == 0, rc
            launch_plan[ni] = nb.last_launch()[:2]

    import ctypes as _C
    lib.gpunb_sort_count.restype = _C.c_longlong
    sort_counter = {"timed": 0}

    def timed_steps(k, precision, graphs=False, timing=True):
        """k steps, each bracketed by CUDA events on the library's stream.
        graphs: replay each call shape as a CUDA graph (gpunb_set_graphs);
        timing: per-pair-kernel events as well (calls then run without graphs)."""
        nb.set_precision(precision)
        lib.gpunb_set_graphs(1 if graphs else 0)
        for _ in range(args.warmup):
            dev_step()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        lib.gpunb_set_timing(1 if timing else 0)
        evs = []
        s0 = lib.gpunb_sort_count()
        for _ in range(k):
            with torch.cuda.stream(stream):    # L2 flush between steps, on the timed
                flush.zero_()                  # stream before its start event (untimed)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            dev_step()
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        sort_counter["timed"] = lib.gpunb_sort_count() - s0
        kt = nb.kernel_times(max_n=64 * k + 64) if timing else []
        lib.gpunb_set_timing(0)
        lib.gpunb_set_graphs(0)
        if dist:
            dist.barrier()
        ms = [a.elapsed_time(b) for a, b in evs]
        return ms, kt

    # ---- split-precision product path, device-resident -------------------
    clocks = Clocks(local)
    clocks.start()
    t_wall = time.perf_counter()
    ms, _ = timed_steps(args.steps, "split", graphs=True, timing=False)
    sorts_timed = sort_counter["timed"]   # j-set re-orderings in the timed steps
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    step_ms = float(sum(ms) / len(ms))
    # the same steps without graphs, with per-pair-kernel events (roofline)
    kt_steps = max(4, min(args.steps, 16))
    ms_nograph, kt = timed_steps(kt_steps, "split", graphs=False, timing=True)
    if dist:
        t = torch.tensor([step_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        step_ms = float(t.item())
    pairs_per_step = N * sum(BLOCKS)
    value = ws * pairs_per_step / (step_ms * 1e-3) / 1e9
    # pair-kernel launches of the dominant block (ni = N), in launch order
    kt = np.asarray(kt).reshape(kt_steps, len(BLOCKS))
    big = kt[:, BLOCKS.index(65536)]
    k_ms = float(np.mean(big))
    # every block's pair kernel: duration, pairs/s and the bound that applies
    # (small blocks read each j tile once: 52 B per body from L2/HBM, and are
    # latency-bound; large ones are FP32-bound)
    # roofline of each block: min(FP32 peak / 60 flops, HBM bandwidth / j bytes per
    # pair), the j tiles read once per i-tile (at most 128 i per tile pass)
    per_block = {}
    fp32_gp = fp32_peak_tflops(gpu_info()[1], clk.get("sm_max_mhz") or 2070.0) * 1e12 / \
        FLOPS_PER_PAIR / 1e9
    for q, ni in enumerate(BLOCKS):
        bm = float(np.mean(kt[:, q]))
        gp = ni * N / (bm * 1e-3) / 1e9
        hbm_gp = hbm_gbs() / (TILE_BYTES_PER_BODY / min(ni, 128))
        bound_gp = min(fp32_gp, hbm_gp)
        per_block[str(ni)] = {"kernel_ms": bm, "gpairs_s": gp,
                              "frac_fp32_nominal": gp / fp32_gp,
                              "roofline_gpairs_s": bound_gp,
                              "roofline": "fp32" if fp32_gp <= hbm_gp else "hbm",
                              "frac_of_roofline": gp / bound_gp,
                              "bound": "fp32" if ni >= 1024 else "latency (j set read once)"}
    pairs_big = 65536 * N
    achieved_tflops = pairs_big * FLOPS_PER_PAIR / (k_ms * 1e-3) / 1e12
    name, n_sm = gpu_info()
    peak_mhz = clk.get("sm_max_mhz") or 2070.0
    peak = fp32_peak_tflops(n_sm, peak_mhz)
    load_mhz = clk.get("sm_mhz") or peak_mhz
    # measured FP32 throughput of this device (packed FMA chains, the pair
    # loop's instruction), after the timed region
    import ctypes as _C
    lib.gpunb_fp32_peak.argtypes = [_C.POINTER(_C.c_float), _C.POINTER(_C.c_float)]
    lib.gpunb_fp32_peak.restype = _C.c_int
    _tf, _ms = _C.c_float(0), _C.c_float(0)
    peak_meas = float(_tf.value) if lib.gpunb_fp32_peak(_C.byref(_tf), _C.byref(_ms)) == 0 \
        else None

    # ---- accuracy of the split kernel against the FP64 kernel ------------
    nb.set_precision("split")
    dev_step()
    torch.cuda.synchronize()
    plan_split = dict(launch_plan)   # the split kernel's shapes (the FP64 pass follows)
    res_split = {ni: (blk[ni]["acc"].cpu().numpy().copy(), blk[ni]["jrk"].cpu().numpy().copy(),
                      blk[ni]["pot"].cpu().numpy().copy()) for ni in (1024, 16384)}
    fp64_ms, fp64_kt = timed_steps(max(1, args.fp64_steps), "fp64")
    fp64_value = ws * pairs_per_step / (float(np.mean(fp64_ms)) * 1e-3) / 1e9
    errs = {}
    for ni in (1024, 16384):
        a64 = blk[ni]["acc"].cpu().numpy(); j64 = blk[ni]["jrk"].cpu().numpy()
        p64 = blk[ni]["pot"].cpu().numpy()
        a, j, p = res_split[ni]
        ea = np.linalg.norm(a - a64, axis=1) / np.linalg.norm(a64, axis=1)
        ej = np.linalg.norm(j - j64, axis=1) / np.linalg.norm(j64, axis=1)
        ep = np.abs(p - p64) / np.abs(p64)
        errs[str(ni)] = {"acc_p99": float(np.percentile(ea, 99)), "acc_max": float(ea.max()),
                         "jrk_p99": float(np.percentile(ej, 99)), "jrk_max": float(ej.max()),
                         "pot_max": float(ep.max())}
    fp64_big = np.asarray(fp64_kt).reshape(-1, len(BLOCKS))[:, BLOCKS.index(65536)]
    # the same step in double-float arithmetic (gpunb_set_precision(2)), against the FP64 kernel
    res_fp64 = {ni: (blk[ni]["acc"].cpu().numpy().copy(), blk[ni]["jrk"].cpu().numpy().copy(),
                     blk[ni]["pot"].cpu().numpy().copy()) for ni in (1024, 16384)}
    df_ms, df_kt = timed_steps(1, "double_float")
    df_value = ws * pairs_per_step / (float(np.mean(df_ms)) * 1e-3) / 1e9
    df_big = np.asarray(df_kt).reshape(-1, len(BLOCKS))[:, BLOCKS.index(65536)]
    df_errs = {}
    for ni in (1024, 16384):
        a64, j64, p64 = res_fp64[ni]
        a = blk[ni]["acc"].cpu().numpy(); j = blk[ni]["jrk"].cpu().numpy()
        p = blk[ni]["pot"].cpu().numpy()
        df_errs[str(ni)] = {
            "acc_max": float((np.linalg.norm(a - a64, axis=1) / np.linalg.norm(a64, axis=1)).max()),
            "jrk_max": float((np.linalg.norm(j - j64, axis=1) / np.linalg.norm(j64, axis=1)).max()),
            "pot_max": float((np.abs(p - p64) / np.abs(p64)).max())}

    # ---- end to end through the C ABI with host arrays --------------------
    nb.set_precision("split")
    hin = {ni: (h2[acts[ni]].copy(), c.dtr[acts[ni]].copy(), c.x[acts[ni]].copy(),
                c.v[acts[ni]].copy()) for ni in BLOCKS}
    outs = {}

    def host_step():
        for ni in BLOCKS:
            nb.send(c.m, c.x, c.v)
            outs[ni] = nb.regf(*hin[ni], LMAX, NNBMAX, out=outs.get(ni))

    def host_steps(graphs):
        lib.gpunb_set_graphs(1 if graphs else 0)   # each call shape replayed as a graph
        for _ in range(args.warmup):
            host_step()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            host_step()
        dt = (time.perf_counter() - t0) / args.steps
        lib.gpunb_set_graphs(0)
        return dt

    e2e_nograph_s = host_steps(False)
    e2e_s = host_steps(True)
    if dist:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    h2d = sum(56 * N + 64 * ni for ni in BLOCKS)
    d2h = sum(60 * ni + 4 * int(np.maximum(outs[ni].list[:, 0], 0).sum()) for ni in BLOCKS)

    batched = None
    if not args.no_batched:
        batched = batched_leg(lib, dev, stream, steps=args.steps, warmup=args.warmup)

    nb.close()
    irr = irr_check = None
    if not args.no_irregular:
        lists_by_particle = np.zeros_like(outs[65536].list)
        lists_by_particle[acts[65536]] = outs[65536].list
        irr, irr_check = irregular_leg(c, h2, lists_by_particle)
    pot, pot_result = potential_leg(c)
    king = king_check = king_cpu = None
    if not args.no_large:
        king, king_check, king_cpu = king1m_leg(lib, dev, stream, n_sm, peak_mhz)
    rsp = rs_predictor_leg(dev)

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu, _ = cpu_baseline(c, acts)
        cpu.update(cpu_side_checks(c, irr_check, pot_result))
        parity = {"bound": "per particle |dQ| <= 1e-6 max(|Q|, sum_j |q_ij| / 8) for force and "
                           "jerk, |dpot| <= 1e-6 |pot|; plain relative errors beside it",
                  "plummer65536_ni16384": oracle_parity(
                      "Plummer N=65536 ni=16384", c.m, c.x, c.v, h2, c.dtr, acts[16384],
                      res_split[16384], LMAX, NNBMAX)}
        if king is not None:
            parity["king1m_ni16384"] = oracle_parity(*king_check, rows=256)
            king["cpu_baseline"] = king_cpu_block(*king_cpu)

    # the library's own kernels: per send copy and pack, plus bbox and Morton
    # keys when the send re-orders the j-set; per regf prep, pair kernel,
    # merge, two scans, gather, offsets, plus the Morton key kernel of the
    # i-ordering when ni >= 256.  The Morton sorts are CUB radix sorts: 6
    # launches per j-set re-ordering, 6 per i-ordering of 16384 or 65536
    # bodies and 1 for 1024 (the launch list in profiles/).
    own = args.steps * (2 * len(BLOCKS) + 7 * len(BLOCKS) + sum(ni >= 256 for ni in BLOCKS)) \
        + 2 * sorts_timed
    cub = args.steps * 13 + 6 * sorts_timed
    line = {
        "metric": METRIC, "value": value, "unit": "Gpairs/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "ms_per_step_without_graphs": float(np.mean(ms_nograph)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Plummer sphere, Kroupa IMF, Henon units)",
        "config": config(ws),
        "impl_detail": {"precision": "split FP32 (double-single positions)",
                        "launch": "device entry points replayed as CUDA graphs, one per call "
                                  "shape"},
        "fp64": {"value": fp64_value, "unit": "Gpairs/s",
                 "kernel_ms_ni65536": float(np.mean(fp64_big)),
                 "speedup_split_over_fp64_kernel": float(np.mean(fp64_big)) / k_ms,
                 "achieved_tflops_60_flops_per_pair":
                     pairs_big * FLOPS_PER_PAIR / (float(np.mean(fp64_big)) * 1e-3) / 1e12,
                 "fp64_peak_tflops": fp64_peak_tflops(n_sm, peak_mhz),
                 "frac_fp64_peak": pairs_big * FLOPS_PER_PAIR /
                     (float(np.mean(fp64_big)) * 1e-3) / 1e12 / fp64_peak_tflops(n_sm, peak_mhz)},
        "rel_err_vs_fp64_kernel": errs,
        "double_float": {"value": df_value, "unit": "Gpairs/s",
                         "kernel_ms_ni65536": float(np.mean(df_big)),
                         "speedup_over_fp64_kernel": float(np.mean(fp64_big)) / float(np.mean(df_big)),
                         "max_rel_err_vs_fp64_kernel": df_errs,
                         "note": "gpunb_set_precision(2): every pair in double-float arithmetic "
                                 "on the FP32 pipe"},
        "pair_kernel_per_block": per_block,
        "launch_plan_per_block": {str(ni): {"variant": v, "splits": sp_}
                                  for ni, (v, sp_) in plan_split.items()},
        "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved_tflops / peak,
                     "frac_at_load_clock": achieved_tflops / fp32_peak_tflops(n_sm, load_mhz),
                     "peak_measured_fp32": peak_meas,
                     "frac_of_measured_fp32": (achieved_tflops / peak_meas) if peak_meas else None,
                     "traffic": read_traffic(),
                     "kernel": "regf_ds_kernel (ni=65536 block)",
                     "kernel_ms": k_ms, "flops_per_pair": FLOPS_PER_PAIR,
                     "peak_source": f"nominal FP32: {n_sm} SMs x 128 lanes x 2 x {peak_mhz:.0f} MHz"
                                    " (MEASURED_PEAKS.json has no FP32 entry)"},
        "e2e": {"value": ws * pairs_per_step / e2e_s / 1e9, "unit": "Gpairs/s",
                "value_without_graphs": ws * pairs_per_step / e2e_nograph_s / 1e9,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": own,
        "library_launches": {"cub_radix_sort": cub},
        "j_set_reorderings": {"timed_sends": args.steps * len(BLOCKS), "reorderings": sorts_timed,
                              "interval": RESORT_EVERY},
        "clocks": clk,
        "wall_s_timed_region": t_wall,
        "device": name,
    }
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if parity is not None:
        line["parity_vs_fp64_oracle"] = parity
    if batched is not None:
        line["batched_clusters"] = batched
    if king is not None:
        line["king1m"] = king
    if irr is not None:
        line["irregular"] = irr
    line["potential"] = pot
    line["rs_predictor_inference"] = rsp
    if args.tune_save:
        lib.gpunb_tune_save(args.tune_save.encode())
    if rank == 0:
        print(json.dumps(line, default=_jsonable), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
