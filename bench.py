#!/usr/bin/env python
"""TOF list-mode OSEM throughput on the clinical-size workload.

Workload (one "step" = one full OSEM iteration = 10 subsets over all events):
  scanner  424/444 mm radii, 48 blocks/ring of 13 x 13 crystals (4 mm), 4 block rings
           (32,448 crystals); TOF 530 ps FWHM (sigma 33.7 mm along the LOR), Gaussian truncated at
           3 sigma; LORs float32 (N, 7), TOF column in mm
  events   2e7, seeded synthetic: water-ellipsoid body (30 x 20 x 100 cm axes) with 0..40 random
           hot/cold ellipsoids (contrast 0.2..8), isotropic emission, hits snapped to crystals
  image    200 x 200 x 109 float32 at 2.04 x 2.04 x 2.03 mm; sensitivity image precomputed on the
           GPU from all 1.05e9 ordered crystal pairs (timed separately, reported as emap_s)
  update   MlemFullTof's rule per subset (div_no_nan(y, p + 1e-5), x * bp / emap) with the
           sensitivity scaled by 1/n_subsets
Metric: LOR-voxel updates/s = (projector + backprojector (LOR, voxel) visits per iteration) /
seconds per iteration; visits are counted exactly by srf_count_pairs.

--impl reference runs the reference's CPU arithmetic (the oracle's restatement of
srfnef's Siddon device functions, with all host threads) on a bounded sample of the same
workload and reports the same metric.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TOF OSEM s/iter & LOR-voxel updates/s on 1 GB300 vs plain, rel L2 err ≤1e-5"
UNIT = "LOR-voxel updates/s"
FALLBACK_HBM_GBS = 6800.0
# DRAM bytes (read + write) of one k_osem_subset launch of this workload (2e6 TOF LORs of an
# interleaved subset, clinical image), from ncu: profiles/k_osem_subset_tof_clinical_2M_lors.txt
NCU_TRAFFIC_SUBSET = 187_686_144


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--events", type=float, default=2e7)
    ap.add_argument("--subsets", type=int, default=10)
    ap.add_argument("--nsigma", type=float, default=3.0)
    ap.add_argument("--lanes", type=int, default=32)
    ap.add_argument("--cpu-sample", type=int, default=400000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--seed", type=int, default=20250101)
    ap.add_argument("--workload", default="clinical",
                    choices=["clinical", "batched", "components", "surrogate", "profile", "autograd",
                             "mlem_small", "conv"],
                    help="clinical: the TOF OSEM headline; batched: 64 uneven studies; "
                         "components: every kernel of the path against the CPU oracle; "
                         "surrogate: learned scatter estimate against SSS (time, sinogram and "
                         "OSEM image agreement); profile: subset steps only, the case ncu captures; "
                         "autograd: differentiable projector, 8 images, forward + backward; "
                         "mlem_small: non-TOF MLEM, 1e5 events, 640-crystal scanner, 64x64x16; "
                         "conv: the surrogate's full-resolution 3-D convolutions in each kernel mode")
    ap.add_argument("--held-out", type=int, default=20, help="surrogate: held-out phantoms timed")
    ap.add_argument("--studies", type=int, default=64)
    ap.add_argument("--autotune", action="store_true", help="tune lanes/slabs per lane first")
    return ap.parse_args()


def workload_config(a):
    return {
        "workload": "tof_listmode_osem_clinical",
        "events": int(a.events), "image": [200, 200, 109], "voxel_mm": [2.04, 2.04, 2.03],
        "crystals": 32448, "subsets": a.subsets, "tof_fwhm_ps": 530.0, "tof_nsigma": a.nsigma,
        "subset_order": "interleaved: event i in subset i mod subsets (OsemFullTof subsets='interleaved')",
        "step": "one full OSEM iteration (all subsets)",
        "l2": "inputs larger than L2 (LOR stream 560 MB per iteration)",
        "lanes_per_lor": a.lanes,
    }


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.path = None
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(gpu_index)], stdout=self.f, stderr=subprocess.DEVNULL)
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
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(a):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if a.impl == "gb300" else "gloo"
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, ws, device=None):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(v, ws, device=None):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------- CPU (oracle) timing

def cpu_sample_rate(lors_np, x_np, ic, tof, nsigma, threads):
    """(pairs per second, pairs, seconds, p, bp) of one fused subset pass (projection p, ratio,
    backprojection bp) of the oracle over lors_np."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import oracle as O
    O.build()
    kw = dict(tof=True, tof_bin=tof[0], tof_sigma2=tof[1], tof_nsigma=nsigma, threads=threads)
    t0 = time.perf_counter()
    p, n1 = O.trace(lors_np, ic.shape, ic.center, ic.size, O.RULES_PROJ, O.GATHER, image=x_np, **kw)
    r = O.ratio(np.ones(len(p), np.float32), p, "full_tof")
    bp, n2 = O.trace(lors_np, ic.shape, ic.center, ic.size, O.RULES_BACK, O.SCATTER, values=r, **kw)
    dt = time.perf_counter() - t0
    return (n1 + n2) / dt, n1 + n2, dt, p, bp


def subset_parity(st_x, samp_dev, x_np, p_ref, bp_ref, ic, tof, nsigma, dev):
    """The GPU subset step on the oracle's sample and image: relative L2 of x * bp (the update
    with a unit sensitivity) against the oracle's, and the FP64 sums y log(p + 1e-5) of both."""
    import numpy as np
    import torch
    from srf_gb300 import kernels
    from srf_gb300._lib import SRF_RATIO_DIV_NO_NAN
    chk = kernels.SubsetState(ic.shape, ic.center, ic.size, dev, x0=st_x)
    chk.subset(samp_dev, None, rule=SRF_RATIO_DIV_NO_NAN, eps=1e-5, tof=tof, tof_nsigma=nsigma,
               track_loglik=True)
    chk.update(kernels.xfast(torch.ones(ic.shape, device=dev)), guard_zero=True)
    got = chk.x.contiguous().cpu().numpy().astype(np.float64)
    want = x_np.astype(np.float64) * bp_ref.astype(np.float64)
    den = (p_ref + np.float32(1e-5)).astype(np.float64)
    ll_ref = float(np.log(den[den > 0]).sum())
    ll_gpu = float(chk.loglik.item())
    return {"events": int(samp_dev.shape[0]),
            "rel_l2_update": float(np.linalg.norm(got - want) / np.linalg.norm(want)),
            "loglik_data_term_gpu": ll_gpu, "loglik_data_term_oracle": ll_ref,
            "loglik_rel_diff": abs(ll_gpu - ll_ref) / max(abs(ll_ref), 1e-300),
            "tolerance": 1e-5}


def l2_peaks(dev):
    """Best-case L2 throughput for 4-byte words on this GPU (srf_calib_l2): loads in GB/s and
    reductions (red.add.f32) per second over a 32 MB L2-resident buffer, CUDA-event timed."""
    import torch
    from srf_gb300._lib import call, i32, i64, ptr, stream_ptr
    from srf_gb300 import _lib
    n = 8 << 20
    buf = torch.zeros(n, dtype=torch.float32, device=dev)
    sink = torch.zeros(int(_lib.load().srf_calib_sink_size()), dtype=torch.float32, device=dev)
    s = stream_ptr(dev)
    stream = torch.cuda.current_stream(dev)
    out = {}
    for mode, reps, key in ((0, 40, "read_gbps"), (1, 20, "red_per_s")):
        call("srf_calib_l2", ptr(buf), i64(n), i32(reps), i32(mode), ptr(sink), s)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call("srf_calib_l2", ptr(buf), i64(n), i32(reps), i32(mode), ptr(sink), s)
        e1.record(stream)
        torch.cuda.synchronize()
        sec = e0.elapsed_time(e1) / 1000.0
        out[key] = (n * reps * 4 / sec / 1e9) if mode == 0 else (n * reps / sec)
    return out


def make_workload(a, device, rank):
    import torch
    from srf_gb300 import synth
    sc, ic = synth.scanner_clinical(), synth.image_clinical()
    act = synth.phantom_body(ic, seed=a.seed + 7, device=device)
    lors = synth.sample_events(sc, ic, act, int(a.events), seed=a.seed + rank, tof_fwhm_ps=530.0,
                               device=device)
    return sc, ic, act, lors


def run_reference(a, ws, rank):
    """Reference arm: the reference's Siddon arithmetic on the host cores (oracle port)."""
    if rank != 0:
        return
    import numpy as np
    import torch
    from srf_gb300 import synth
    sc, ic = synth.scanner_clinical(), synth.image_clinical()
    n = int(a.cpu_sample)
    act = synth.phantom_body(ic, seed=a.seed + 7)
    lors = synth.sample_events(sc, ic, act, n, seed=a.seed, tof_fwhm_ps=530.0).numpy()
    x = np.ones(ic.shape, dtype=np.float32)
    tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    threads = os.cpu_count() or 1
    for _ in range(a.warmup):
        cpu_sample_rate(lors[: max(1000, n // 20)], x, ic, tof, a.nsigma, threads)
    rates, secs = [], []
    for _ in range(a.steps):
        r, pairs, dt, _, _ = cpu_sample_rate(lors, x, ic, tof, a.nsigma, threads)
        rates.append(r)
        secs.append(dt)
    val = statistics.median(rates)
    sample = (f"{n} of {int(a.events)} events per step: one TOF subset pass (projection, ratio, "
              f"backprojection) of the oracle restatement of srfnef's Siddon device functions")
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000 * statistics.median(secs),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": workload_config(a),
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_batched(a, ws, rank, local):
    """64 independent TOF studies (events log-uniform in [1e5, 5e6], images 64^3, 96x96x64,
    128x128x80 or 160x160x80 at 2, 3 or 4 mm), 4 subsets x 2 iterations each, on the clinical
    scanner: every study alone (two kernels per subset step) and all studies together (two batch
    kernels per subset step, one iteration captured in a CUDA graph and replayed)."""
    import numpy as np
    import torch
    from srf_gb300 import _lib, autotune, kernels, synth
    from srf_gb300._lib import SRF_RATIO_DIV_NO_NAN
    from srf_gb300.geometry import ImageConfig, block_full_crystal_table
    from srf_gb300.studies import Study, StudyBatch
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.load()
    sc = synth.scanner_clinical()
    tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    rng = np.random.default_rng(a.seed + 17 * rank)
    shapes = [(64, 64, 64), (96, 96, 64), (128, 128, 80), (160, 160, 80)]
    n_sub, n_iter = 4, 2
    table = torch.as_tensor(block_full_crystal_table(sc), device=dev)
    emaps = {}
    studies, meta = [], []
    t0 = time.perf_counter()
    for j in range(a.studies):
        shape = shapes[int(rng.integers(0, 4))]
        vox = float(rng.choice([2.0, 3.0, 4.0]))
        n = int(round(math.exp(rng.uniform(math.log(1e5), math.log(5e6)))))
        ic = ImageConfig(list(shape), [0.0, 0.0, 0.0], [s * vox for s in shape])
        key = (shape, vox)
        if key not in emaps:
            emaps[key] = kernels.emap_block_full(table, sc.nb_blocks_per_ring, ic.shape, ic.center, ic.size)
        act = synth.phantom_body(ic, seed=a.seed + j, device=dev)
        lors = synth.sample_events(sc, ic, act, n, seed=a.seed + 1000 + j, tof_fwhm_ps=530.0, device=dev)
        emx = kernels.xfast(emaps[key] / n_sub)
        studies.append(Study(lors, ic.shape, ic.center, ic.size, emx))
        meta.append({"shape": list(shape), "voxel_mm": vox, "events": n})
    setup_s = time.perf_counter() - t0
    tuned = None
    if a.autotune:
        big = max(range(len(studies)), key=lambda j: studies[j].lors.shape[0])
        s0 = studies[big]
        tuned = autotune.tune(s0.lors[: 1 << 20].contiguous(), s0.shape, s0.center, s0.size, tof,
                              a.nsigma, reps=2, cache=None)
    batch = StudyBatch(studies, n_sub, tof, tof_nsigma=a.nsigma, seed=a.seed)
    visits = []
    for st in studies:
        f = kernels.count_pairs(st.lors, st.shape, st.center, st.size, rules=0, tof=tof, tof_nsigma=a.nsigma)
        b = kernels.count_pairs(st.lors, st.shape, st.center, st.size, rules=1, tof=tof, tof_nsigma=a.nsigma)
        visits.append(f + b)
    stream = torch.cuda.current_stream(dev)

    def ev():
        return torch.cuda.Event(enable_timing=True)

    # every study alone
    per_study = []
    for st in studies:
        per = st.lors.shape[0] // n_sub

        def one_iter():
            for k in range(n_sub):
                st.state.subset(st.lors[k * per:(k + 1) * per], None, rule=SRF_RATIO_DIV_NO_NAN,
                                eps=1e-5, tof=tof, tof_nsigma=a.nsigma)
                st.state.update(st.emap, guard_zero=True)
        one_iter()
        e0, e1 = ev(), ev()
        e0.record(stream)
        for _ in range(n_iter):
            one_iter()
        e1.record(stream)
        torch.cuda.synchronize()
        per_study.append(e0.elapsed_time(e1) / n_iter / 1000.0)
    # all together: eager, then graph replay
    batch.reset()
    batch.iteration()
    torch.cuda.synchronize()
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(n_iter):
        batch.iteration()
    e1.record(stream)
    torch.cuda.synchronize()
    eager_s = e0.elapsed_time(e1) / n_iter / 1000.0
    reps = max(a.steps, n_iter)

    def graph_time(concurrent):
        batch.reset()
        batch.capture(concurrent=concurrent)
        batch.reset()
        e0, e1 = ev(), ev()
        e0.record(stream)
        for _ in range(reps):
            batch.replay()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps / 1000.0

    clocks = Clocks(local)
    graph_persistent_s = graph_time(False)
    graph_concurrent_s = graph_time(True)
    clk = clocks.stop()
    graph_s = min(graph_persistent_s, graph_concurrent_s)
    total_visits = float(sum(visits))
    if rank == 0:
        line = {
            "metric": "batched TOF OSEM s/iter (64 uneven studies) & LOR-voxel updates/s",
            "value": total_visits / graph_s, "unit": UNIT, "n_gpus": ws, "steps": reps,
            "warmup": 1, "ms_per_step": graph_s * 1000.0, "s_per_iter_all_studies": graph_s,
            "s_per_iter_graph_persistent_batch_kernel": graph_persistent_s,
            "s_per_iter_graph_concurrent_study_chains": graph_concurrent_s,
            "s_per_iter_all_studies_eager_batch": eager_s,
            "s_per_iter_sum_of_single_studies": float(sum(per_study)),
            # every study at the best single-study visit rate: what no batching can beat
            "s_per_iter_ceiling_best_single_rate": total_visits / max(v / t for v, t in zip(visits, per_study)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded phantoms per study)",
            "config": {"workload": "batched_uneven_studies", "studies": len(studies),
                       "subsets": n_sub, "iterations": n_iter, "tof_nsigma": a.nsigma,
                       "events_total": int(sum(m["events"] for m in meta)),
                       "setup_s": setup_s, "autotune": tuned},
            "per_study": [dict(m, s_per_iter=t, visits_per_iter=v) for m, t, v in zip(meta, per_study, visits)],
            "gpu_launches": (2 * n_sub if graph_s == graph_persistent_s else 2 * n_sub * len(studies)) * reps,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)


def run_conv(a, ws, rank, local):
    """The scatter U-Net's full-resolution convolutions (batch 1, 28 x 28 x 160 voxels, Cin 16 / 32 /
    96 -> Cout 32, BF16 with FP32 accumulation) in each srf_conv3d_fwd kernel mode: 0 mma.sync,
    1 tcgen05 K-step tiles (the default), 2 / 3 tcgen05 on halo tiles loaded by cp.async / TMA. CUDA events, best of
    --steps after --warmup; the kernel each mode took is reported (srf_conv_last_path)."""
    import ctypes
    import numpy as np
    import torch
    from srf_gb300 import _lib
    from srf_gb300._lib import call, i32, ptr, stream_ptr
    from srf_gb300.surrogate import act
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.load()
    s = stream_ptr(dev)
    rng = np.random.default_rng(a.seed)
    shape = (1, 28, 28, 160)
    names = {0: "mma.sync 64x64", 1: "mma.sync 128x32", 2: "tcgen05 K-step", 3: "tcgen05 TMA halo",
             4: "mma.sync split-K", 5: "tcgen05 cp.async halo"}
    layers = []
    try:
        for cin, cout in ((16, 32), (32, 32), (96, 32)):
            x = torch.as_tensor(rng.standard_normal(shape + (cin,)).astype(np.float32)).to(torch.bfloat16).to(dev)
            w = (torch.as_tensor(rng.standard_normal((cout, 27, cin)).astype(np.float32)) * 0.1).to(torch.bfloat16).to(dev)
            b = torch.zeros(cout, device=dev)
            y = torch.empty(shape + (cout,), dtype=torch.bfloat16, device=dev)
            flops = 2.0 * 27 * cin * cout * float(np.prod(shape))
            rec = {"cin": cin, "cout": cout, "gflop": flops / 1e9}
            for mode in (0, 1, 2, 3):
                call("srf_set_conv_tc", i32(mode))
                run = lambda: call("srf_conv3d_fwd", ptr(x), act(x), i32(cin), ptr(w), ptr(b), i32(cout), i32(1),
                                   ptr(y), act(y), None, s)
                for _ in range(max(a.warmup, 1)):
                    run()
                torch.cuda.synchronize()
                best = float("inf")
                for _ in range(a.steps):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record()
                    run()
                    e1.record()
                    torch.cuda.synchronize()
                    best = min(best, e0.elapsed_time(e1))
                path = ctypes.c_int32(-1)
                call("srf_conv_last_path", ctypes.byref(path))
                rec[f"mode{mode}"] = {"us": 1000 * best, "tflops": flops / (best * 1e-3) / 1e12,
                                      "kernel": names.get(path.value, str(path.value))}
            layers.append(rec)
    finally:
        call("srf_set_conv_tc", i32(1))
    if rank == 0:
        tot = {m: sum(l[f"mode{m}"]["us"] for l in layers) for m in (0, 1, 2, 3)}
        print(json.dumps({
            "metric": "full-resolution 3-D convolution time of the scatter U-Net (three layers)",
            "value": tot[1], "unit": "us", "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulation)",
            "data": "synthetic (seeded)", "config": {"workload": "conv", "grid": list(shape[1:]), "batch": 1},
            "layers": layers, "total_us_by_mode": tot, "gpu_launches": 12 * (a.steps + max(a.warmup, 1))}), flush=True)


def run_mlem_small(a, ws, rank, local):
    """Non-TOF list-mode MLEM on the 640-crystal scanner (99 mm inner radius, 16 blocks of
    10 x 4 crystals, 4 block rings): 1e5 seeded events of the water cylinder with six hot spheres
    (snapped to crystal centres), image 64 x 64 x 16 at 2 mm, sensitivity image over all 409,600
    ordered crystal pairs, 10 iterations of MlemFull's update (div_no_nan(y, p), x * bp / emap).

    One step = one MLEM iteration with the inputs resident. The end-to-end leg is the whole job
    through the drop-in, MlemFull(10, ...)() on numpy inputs: sensitivity image, 10 iterations,
    image back as numpy. The CPU baseline is the oracle doing the same job on one thread; the
    GPU job's image is compared with the oracle's."""
    import numpy as np
    import torch
    import srf_gb300 as nef
    from srf_gb300 import _lib, kernels, synth
    from srf_gb300._lib import SRF_RATIO_DIV_NO_NAN
    from srf_gb300.geometry import block_full_crystal_table
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.load()
    sc, ic = synth.scanner_small(), synth.image_small()
    n_ev, n_iter = 100_000, 10
    act = synth.phantom_cylinder(ic, device=dev)
    lors = synth.sample_events(sc, ic, act, n_ev, seed=a.seed + rank, tof_fwhm_ps=530.0, device=dev)
    lors6 = lors[:, :6].contiguous()
    stream = torch.cuda.current_stream(dev)
    table = torch.as_tensor(block_full_crystal_table(sc), device=dev)
    emap = kernels.emap_block_full(table, sc.nb_blocks_per_ring, ic.shape, ic.center, ic.size)
    p_fwd = kernels.count_pairs(lors6, ic.shape, ic.center, ic.size, rules=0)
    p_bwd = kernels.count_pairs(lors6, ic.shape, ic.center, ic.size, rules=1)
    st = kernels.SubsetState(ic.shape, ic.center, ic.size, dev)

    def iteration():
        st.subset(lors6, None, rule=SRF_RATIO_DIV_NO_NAN, eps=0.0)
        st.update(emap, guard_zero=True)

    for _ in range(a.warmup):
        iteration()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    barrier(ws)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(a.steps):
        iteration()
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms_step = max_over_ranks(e0.elapsed_time(e1) / a.steps, ws, dev)
    upd = float(p_fwd + p_bwd)
    # the whole job through the drop-in, numpy in and out
    y_np = np.ones(n_ev, np.float32)
    l_np = lors6.cpu().numpy()
    lm = nef.Listmode(y_np, nef.Lors(l_np))
    job = lambda: nef.MlemFull(n_iter, ic, sc, lm, None, None, None, None)()
    job()
    torch.cuda.synchronize()
    reps = 5
    t0 = time.perf_counter()
    for _ in range(reps):
        out = job()
    torch.cuda.synchronize()
    job_s = (time.perf_counter() - t0) / reps
    cpu = parity = None
    if rank == 0 and not a.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        O.build()
        t0 = time.perf_counter()
        em_ref = O.emap_block_full(block_full_crystal_table(sc), sc.nb_blocks_per_ring, ic.shape,
                                   ic.center, ic.size)
        ref = O.mlem(l_np, y_np, em_ref, ic.shape, ic.center, ic.size, n_iter, rule="full")
        cpu_s = time.perf_counter() - t0
        cpu = {"value": n_iter * upd / cpu_s, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": f"the whole job (sensitivity image + {n_iter} iterations) on the oracle, "
                         f"{cpu_s:.2f} s", "job_s": cpu_s}
        parity = {"rel_l2_image": O.rel_l2(out.data, ref),
                  "rel_l2_emap": O.rel_l2(emap.contiguous().cpu().numpy(), em_ref), "tolerance": 1e-5}
    if rank == 0:
        print(json.dumps({
            "metric": "non-TOF list-mode MLEM s/iter & LOR-voxel updates/s (640-crystal scanner)",
            "value": upd / (ms_step / 1000.0), "unit": UNIT, "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_step, "s_per_iter": ms_step / 1000.0,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded cylinder phantom, events snapped to crystals)",
            "config": {"workload": "mlem_nontof_small", "events": n_ev, "image": ic.shape,
                       "voxel_mm": 2.0, "crystals": int(sc.nb_crystals), "iterations": n_iter,
                       "emap_lors": int(sc.nb_crystals) ** 2,
                       "l2": "inputs L2-resident (2.4 MB of LORs), not flushed"},
            "updates_per_iter": upd, "pairs_fwd": p_fwd, "pairs_bwd": p_bwd,
            "job_s": job_s,
            "e2e": {"value": n_iter * upd / job_s, "unit": UNIT, "h2d_bytes_per_step": int(l_np.nbytes + y_np.nbytes),
                    "d2h_bytes_per_step": int(np.prod(ic.shape) * 4), "ms_per_step": 1000 * job_s,
                    "path": "srf_gb300.MlemFull(10, ...)() on numpy inputs, sensitivity image included"},
            "cpu_baseline": cpu, "parity": parity, "clocks": clk,
            "gpu_launches": 2 * a.steps}), flush=True)


def run_components(a, ws, rank, local):
    """Each kernel of the path on the clinical geometry, timed with CUDA events (best of 5 after
    a warm-up), beside the CPU oracle on a sample (single thread)."""
    import numpy as np
    import torch
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from srf_gb300 import _lib, kernels, synth
    from srf_gb300.geometry import block_full_crystal_table, EcatIndexToCrystalPos
    from srf_gb300._lib import SRF_RATIO_DIV_NO_NAN
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.load()
    O.build()
    sc, ic = synth.scanner_clinical(), synth.image_clinical()
    act = synth.phantom_body(ic, seed=a.seed + 7, device=dev)
    n = 2_000_000
    lors = synth.sample_events(sc, ic, act, n, seed=a.seed, tof_fwhm_ps=530.0, device=dev)
    lors6 = lors[:, :6].contiguous()
    tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    img = kernels.xfast(act + 0.1)
    img_t = kernels.yfast(img)
    vals = torch.rand(n, device=dev)
    samp = 20000
    l_np, l6_np = lors[:samp].cpu().numpy(), lors6[:samp].cpu().numpy()
    img_np = img.contiguous().cpu().numpy()
    v_np = vals[:samp].cpu().numpy()

    def gpu_ms(fn, reps=5):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    def cpu_s(fn):
        t0 = time.perf_counter()
        fn()
        return time.perf_counter() - t0

    out = {}
    for name, t, rules, ns in (("projection_tof_3sigma", tof, 0, a.nsigma), ("backprojection_tof_3sigma", tof, 1, a.nsigma),
                               ("projection_tof_exact", tof, 0, 0.0), ("backprojection_tof_exact", tof, 1, 0.0),
                               ("projection_nontof", None, 0, 0.0), ("backprojection_nontof", None, 1, 0.0)):
        L = lors if t is not None else lors6
        pairs = kernels.count_pairs(L, ic.shape, ic.center, ic.size, rules=rules, tof=t, tof_nsigma=ns)
        if rules == 0:
            ms = gpu_ms(lambda: kernels.project(L, img, ic.center, ic.size, tof=t, tof_nsigma=ns, image_t=img_t))
        else:
            ms = gpu_ms(lambda: kernels.backproject(L, vals, ic.shape, ic.center, ic.size, tof=t, tof_nsigma=ns))
        kw = dict(tof=True, tof_bin=t[0], tof_sigma2=t[1], tof_nsigma=ns) if t is not None else {}
        Ln = l_np if t is not None else l6_np
        if rules == 0:
            cs = cpu_s(lambda: O.projection(img_np, Ln, ic.shape, ic.center, ic.size, **kw))
        else:
            cs = cpu_s(lambda: O.backprojection(v_np, Ln, ic.shape, ic.center, ic.size, **kw))
        cpu_pairs = pairs * samp / n
        out[name] = {"lors": n, "pairs": pairs, "ms": ms, "pairs_per_s": pairs / (ms / 1e3),
                     "cpu_pairs_per_s": cpu_pairs / cs, "cpu_sample_lors": samp}
    st = kernels.SubsetState(ic.shape, ic.center, ic.size, dev)
    ms = gpu_ms(lambda: st.subset(lors, None, rule=SRF_RATIO_DIV_NO_NAN, eps=1e-5, tof=tof, tof_nsigma=a.nsigma))
    pf = out["projection_tof_3sigma"]["pairs"] + out["backprojection_tof_3sigma"]["pairs"]
    out["osem_subset_fused"] = {"lors": n, "pairs": pf, "ms": ms, "pairs_per_s": pf / (ms / 1e3)}
    em_x = kernels.xfast(torch.ones(ic.shape, device=dev))
    ms = gpu_ms(lambda: st.update(em_x, guard_zero=True))
    out["osem_update"] = {"voxels": int(np.prod(ic.shape)), "ms": ms,
                          "gb_per_s": 8 * 4 * float(np.prod(ic.shape)) / (ms / 1e3) / 1e9}
    table = torch.as_tensor(block_full_crystal_table(sc), device=dev)
    ms = gpu_ms(lambda: kernels.emap_block_full(table, sc.nb_blocks_per_ring, ic.shape, ic.center, ic.size), reps=2)
    m = table.shape[0] // sc.nb_blocks_per_ring
    tnp = table.cpu().numpy()
    p1 = np.repeat(tnp[:m][:40], m, axis=0)
    p2 = np.tile(tnp[5 * m:6 * m], (40, 1))
    cl = np.hstack([p1, p2]).astype(np.float32)
    cs = cpu_s(lambda: O.backprojection(np.ones(len(cl), np.float32), cl, ic.shape, ic.center, ic.size))
    out["emap_block_full"] = {"lors": int(sc.nb_crystals) ** 2, "ms": ms,
                              "lors_per_s": sc.nb_crystals ** 2 / (ms / 1e3), "cpu_lors_per_s": len(cl) / cs}
    # single-scatter simulation: random crystal pairs x scatter points of a 64x64x32 volume
    rng = np.random.default_rng(a.seed)
    cpos = EcatIndexToCrystalPos(sc)(np.arange(sc.nb_crystals)).astype(np.float32)
    n_s = 12 * 12 * 4
    spos = np.stack(np.meshgrid(np.linspace(-250, 250, 12), np.linspace(-250, 250, 12),
                                np.linspace(-80, 80, 4), indexing="ij"), -1).reshape(-1, 3).astype(np.float32)
    em = rng.uniform(0.5, 2.0, (sc.nb_crystals, n_s)).astype(np.float32)
    at = rng.uniform(0.2, 1.0, (sc.nb_crystals, n_s)).astype(np.float32)
    umap = (rng.random((64, 64, 32)) * 0.0096).astype(np.float32)
    np_pairs = 200_000
    pairs = rng.integers(0, sc.nb_crystals, (np_pairs, 2)).astype(np.int32)
    d = lambda x: torch.as_tensor(x).to(dev)
    args = (d(cpos), d(spos), d(em), d(at), d(umap), [600.0, 600.0, 208.0], 624, 48, [1, 13, 13], 350, 650, 0.15)
    ms = gpu_ms(lambda: kernels.sss(d(pairs), *args), reps=3)
    cs = cpu_s(lambda: O.sss(pairs[:2000], cpos, spos, em, at, umap, [600.0, 600.0, 208.0], 624, 48, [1, 13, 13], 350, 650, 0.15))
    out["sss"] = {"pairs": np_pairs, "scatter_points": n_s, "ms": ms,
                  "evals_per_s": np_pairs * n_s / (ms / 1e3), "cpu_evals_per_s": 2000 * n_s / cs}
    ms = gpu_ms(lambda: kernels.snap(lors, sc))
    from srf_gb300.geometry import PetEcatListmodeTrans
    from srf_gb300.data import Listmode, Lors
    cs = cpu_s(lambda: PetEcatListmodeTrans(sc)(Listmode(np.ones(samp, np.float32), Lors(l_np))))
    out["listmode_snap"] = {"events": n, "ms": ms, "events_per_s": n / (ms / 1e3), "cpu_events_per_s": samp / cs}
    ms = gpu_ms(lambda: kernels.lm2sino(lors, None, sc))
    out["lm2sino"] = {"events": n, "ms": ms, "events_per_s": n / (ms / 1e3)}
    mu = kernels.xfast(act * 0.0096)
    ms = gpu_ms(lambda: kernels.attenuation(lors6, mu, ic.center, ic.size))
    out["attenuation_fused"] = {"lors": n, "ms": ms, "lors_per_s": n / (ms / 1e3)}
    if rank == 0:
        print(json.dumps({"metric": "per-kernel throughput, clinical geometry", "workload": "components",
                          "components": out, "cpu_threads": 1, "data": "synthetic"}), flush=True)


def run_profile(a, ws, rank, local):
    """Subset steps of the clinical workload without the sensitivity image and visit counts
    (emap = 1): warmup + steps iterations of n_subsets (subset, update) launch pairs, on the
    headline's interleaved subsets (strided views of the events)."""
    import torch
    from srf_gb300 import _lib, kernels
    from srf_gb300._lib import SRF_RATIO_DIV_NO_NAN
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.load()
    _lib.set_group_lanes(a.lanes)
    sc, ic, act, lors = make_workload(a, dev, rank)
    tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    n_per = lors.shape[0] // a.subsets
    em = torch.ones(ic.shape[::-1], device=dev).permute(2, 1, 0)
    st = kernels.SubsetState(ic.shape, ic.center, ic.size, dev)
    for _ in range(a.warmup + a.steps):
        for k in range(a.subsets):
            st.subset(lors[k:n_per * a.subsets:a.subsets], None, rule=SRF_RATIO_DIV_NO_NAN, eps=1e-5,
                      tof=tof, tof_nsigma=a.nsigma)
            st.update(em, guard_zero=True)
    torch.cuda.synchronize()
    if rank == 0:
        print(json.dumps({"workload": "profile", "events": int(lors.shape[0]), "lors_per_launch": n_per,
                          "subset_launches": (a.warmup + a.steps) * a.subsets}), flush=True)


def run_autograd(a, ws, rank, local):
    """Differentiable projector: a batch of 8 images 128 x 128 x 64 (3.2 mm voxels; seeded random
    ellipsoid mixtures), 5e6 TOF LORs on the clinical scanner, Poisson negative log-likelihood
    against seeded Poisson counts. One step = forward projection of the batch, loss, backward
    (exact adjoint) into the images' gradients; metric = (LOR, voxel) visits of both passes for all
    8 images per second. The same step with the single-image kernels in a loop is timed beside."""
    import torch
    from srf_gb300 import _lib, autograd, kernels, synth
    from srf_gb300.geometry import ImageConfig
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.load()
    _lib.set_group_lanes(a.lanes)
    sc = synth.scanner_clinical()
    ic = ImageConfig([128, 128, 64], [0.0, 0.0, 0.0], [128 * 3.2, 128 * 3.2, 64 * 3.2])
    B = 8
    imgs = torch.stack([synth.phantom_body(ic, seed=a.seed + 100 + b, device=dev) + 0.05 for b in range(B)])
    n_ev = 5_000_000
    lors = synth.sample_events(sc, ic, imgs[0], n_ev, seed=a.seed, tof_fwhm_ps=530.0, device=dev)
    tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    g = torch.Generator(device=dev).manual_seed(a.seed)
    with torch.no_grad():
        p0 = kernels.project_batch(lors, imgs, ic.center, ic.size, tof=tof, tof_nsigma=a.nsigma)
        y = torch.poisson(p0.clamp(min=0) * (5.0 / p0.mean()), generator=g)
    visits = kernels.count_pairs(lors, ic.shape, ic.center, ic.size, rules=0, tof=tof, tof_nsigma=a.nsigma)
    x = (imgs * 0 + 1.0).requires_grad_(True)
    stream = torch.cuda.current_stream(dev)

    def step():
        x.grad = None
        p = autograd.project(x, lors, ic.center, ic.size, tof=tof, tof_nsigma=a.nsigma)
        loss = autograd.poisson_nll(p, y, eps=1e-6)
        loss.backward()
        return loss

    def step_loop():
        loss = 0.0
        for b in range(B):
            xb = x[b].detach().clone().requires_grad_(True)
            p = autograd.project(xb, lors, ic.center, ic.size, tof=tof, tof_nsigma=a.nsigma)
            lb = autograd.poisson_nll(p, y[b], eps=1e-6)
            lb.backward()
            loss = loss + lb.detach()
        return loss

    def timed(f, k):
        for _ in range(max(a.warmup, 3)):
            f()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            f()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k / 1000.0

    clocks = Clocks(local)
    t_batch = timed(step, a.steps)
    clk = clocks.stop()
    t_loop = timed(step_loop, max(2, a.steps // 4))
    total = 2.0 * visits * B
    if rank == 0:
        print(json.dumps({
            "metric": "differentiable TOF projector: forward + adjoint LOR-voxel visits/s (8-image batch)",
            "value": total / t_batch, "unit": "LOR-voxel visits/s", "n_gpus": ws, "steps": a.steps,
            "warmup": max(a.warmup, 3), "ms_per_step": 1000 * t_batch, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded ellipsoid-mixture images, seeded Poisson counts)",
            "config": {"workload": "differentiable_projector", "images": B, "image": ic.shape,
                       "voxel_mm": 3.2, "lors": int(lors.shape[0]), "tof_fwhm_ps": 530.0,
                       "tof_nsigma": a.nsigma, "loss": "Poisson NLL", "visits_per_image": visits},
            "ms_per_step_single_image_loop": 1000 * t_loop, "batch_speedup": t_loop / t_batch,
            "gpu_launches": a.steps * (2 + B), "clocks": clk}), flush=True)


def run_surrogate(a, ws, rank, local):
    """Learned scatter estimate against the single-scatter simulation on held-out phantoms.

    Scatter estimation time, from the emission and mu volumes to the coarse scatter sinogram:
    SSS = preprocessing projections + srf_sss over all 827,424 bins; surrogate = network input
    projections + U-Net forward with its sub-voxel head + the spot-check SSS on 2048 random bins
    and the smooth correction fitted on half of them.
    Agreement: full-sinogram relative L2 on every held-out phantom, and for one study the TOF
    OSEM image with the surrogate's scatter against the image with SSS scatter (and the image
    without scatter correction, for scale)."""
    import torch
    from srf_gb300 import _lib, synth
    from srf_gb300.scatter_sinogram import CoarseGeometry, ScatterStudy, random_phantom, sss_sinogram
    from srf_gb300.surrogate import ScatterSurrogate
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.load()
    geo = CoarseGeometry(synth.scanner_clinical(), device=dev)
    sur = ScatterSurrogate.load(geo)
    stream = torch.cuda.current_stream(dev)

    def timed(f):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0.record(stream)
        r = f()
        e1.record(stream)
        torch.cuda.synchronize()
        return max(e0.elapsed_time(e1) / 1000.0, time.perf_counter() - t0), r

    seeds = [1_000_000 + i for i in range(a.held_out)]
    em, mu = random_phantom(seeds[0], device=dev)
    for _ in range(max(a.warmup, 1)):
        sss_sinogram(geo, em, mu)
        sur.estimate(em, mu)
    t_sss, t_sur, t_net, t_pred, t_spot, errs, spot, fallbacks = [], [], [], [], [], [], [], 0
    cerrs, spot_raw = [], []
    clocks = Clocks(local)
    for sd in seeds:
        em, mu = random_phantom(sd, device=dev)
        ts, ref = timed(lambda: sss_sinogram(geo, em, mu))
        tn, (cest, _) = timed(lambda: sur.estimate(em, mu, fallback=False))
        cerrs.append(float((torch.linalg.vector_norm(cest - ref) / torch.linalg.vector_norm(ref)).item()))
        t_net.append(tn)
        tc, (est, info) = timed(lambda: sur.estimate(em, mu))
        tp, pred = timed(lambda: sur.predict(em, mu))
        tk, _ = timed(lambda: sur.spot_check(em, mu, pred))
        t_pred.append(tp)
        t_spot.append(tk)
        errs.append(float((torch.linalg.vector_norm(pred - ref) / torch.linalg.vector_norm(ref)).item()))
        spot.append(info["spot_rel_l2"])
        spot_raw.append(info["spot_rel_l2_uncorrected"])
        fallbacks += int(info["fallback"])
        t_sss.append(ts)
        t_sur.append(tc)
    clk = clocks.stop()
    # the OSEM image on every held-out phantom: SSS scatter against the corrected network estimate
    # (what the network path gives), and against what the guard returns (SSS on a fallback)
    rel = lambda u, v: float((torch.linalg.vector_norm(u - v) / torch.linalg.vector_norm(v)).item())
    img_net, img_guard, img_none, fb5 = [], [], [], 0
    study = None
    for sd in seeds:
        st_ = ScatterStudy(geo, sd, n_trues=int(min(a.events, 2e6)))
        study = study or st_
        i_sss = st_.reconstruct(st_.sss)
        est, info = sur.estimate(st_.emission, st_.mu, fallback=False)
        e_net = rel(st_.reconstruct(est), i_sss)
        img_net.append(e_net)
        img_guard.append(0.0 if info["spot_rel_l2"] > sur.fallback_tol else e_net)
        img_none.append(rel(st_.x0, i_sss))
        fb5 += int(info["spot_rel_l2"] > 0.05)
    img_sss = study.reconstruct(study.sss)
    img_sur = study.reconstruct(sur.estimate(study.emission, study.mu, fallback=False)[0])
    # the reference's SSS core runs on the CPU (numba); its C restatement (the oracle) on one host
    # core over a 2,000-bin sample of the first held-out phantom, extrapolated to every bin
    cpu_sss = None
    if rank == 0 and not a.no_cpu:
        import numpy as np
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle as O
        from srf_gb300.scatter_sinogram import sss_args, sss_tables
        O.build()
        em0, mu0 = random_phantom(seeds[0], device=dev)
        sumup, atten = sss_tables(geo, em0, mu0, geo.vpos_dev)
        sample = np.ascontiguousarray(geo.pairs[np.random.default_rng(a.seed).choice(geo.n_bins(), 2000, replace=False)])
        t0 = time.perf_counter()
        O.sss(sample, geo.vpos, geo.scatter_points.astype(np.float32), sumup.cpu().numpy(), atten.cpu().numpy(),
              mu0.cpu().numpy(), list(geo.ic.size), *sss_args(geo))
        t_cpu = (time.perf_counter() - t0) * geo.n_bins() / len(sample)
        cpu_sss = {"core_s_estimate": t_cpu, "cores": 1, "kind": "port",
                   "sample": "2000 of 827,424 bins, SSS core only (preprocessing excluded)",
                   "network_path_speedup": None}
    med_sss, med_sur, med_net = statistics.median(t_sss), statistics.median(t_sur), statistics.median(t_net)
    if cpu_sss is not None:
        cpu_sss["network_path_speedup"] = cpu_sss["core_s_estimate"] / med_net
    mean_sss, mean_sur = sum(t_sss) / len(t_sss), sum(t_sur) / len(t_sur)
    if rank == 0:
        print(json.dumps({
            "metric": "scatter estimation speed-up of the learned surrogate path (network + "
                      "concurrent spot-check SSS) over SSS, same sinogram",
            "value": med_sss / med_net, "unit": "x", "n_gpus": ws, "steps": len(seeds),
            "warmup": max(a.warmup, 1), "ms_per_step": 1000 * med_net, "higher_is_better": True,
            "speedup_with_fallbacks": mean_sss / mean_sur,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (network), f32 (SSS)",
            "data": "synthetic (seeded held-out phantoms)",
            "config": {"workload": "scatter_surrogate", "volumes": [64, 64, 32], "bins": geo.n_bins(),
                       "scatter_points": int(geo.scatter_points.shape[0]), "held_out": len(seeds),
                       "spot_check_bins": sur.spot_bins, "fallback_tol": sur.fallback_tol,
                       "params": sur.net.n_params()},
            "sss_s_median": med_sss, "network_path_s_median": med_net,
            "guarded_estimate_s_median": med_sur,
            "predict_s_median": statistics.median(t_pred),
            "spot_check_s_median": statistics.median(t_spot),
            "sinogram_rel_l2_mean": sum(errs) / len(errs), "sinogram_rel_l2_max": max(errs),
            "sinogram_rel_l2_corrected_mean": sum(cerrs) / len(cerrs),
            "sinogram_rel_l2_corrected_max": max(cerrs),
            "spot_rel_l2_mean": sum(spot) / len(spot),
            "spot_rel_l2_uncorrected_mean": sum(spot_raw) / len(spot_raw), "fallbacks": fallbacks,
            "fallbacks_at_5pct_spot": fb5,
            "sss_cpu_reference_port": cpu_sss,
            "osem": {"events": int(study.events.shape[0]), "scatter_fraction": study.sf,
                     "iterations": study.n_iter, "subsets": study.n_sub,
                     "image_rel_l2_surrogate_vs_sss": rel(img_sur, img_sss),
                     "image_rel_l2_uncorrected_vs_sss": rel(study.x0, img_sss),
                     "held_out_image_rel_l2_network_mean": sum(img_net) / len(img_net),
                     "held_out_image_rel_l2_network_max": max(img_net),
                     "held_out_image_rel_l2_guarded_max": max(img_guard),
                     "held_out_image_rel_l2_uncorrected_min": min(img_none)},
            "clocks": clk,
        }), flush=True)


def main():
    a = parse()
    ws, rank, local = dist_setup(a)
    if a.impl == "reference":
        run_reference(a, ws, rank)
        return
    if a.workload == "batched":
        run_batched(a, ws, rank, local)
        return
    if a.workload == "components":
        run_components(a, ws, rank, local)
        return
    if a.workload == "surrogate":
        run_surrogate(a, ws, rank, local)
        return
    if a.workload == "profile":
        run_profile(a, ws, rank, local)
        return
    if a.workload == "autograd":
        run_autograd(a, ws, rank, local)
        return
    if a.workload == "mlem_small":
        run_mlem_small(a, ws, rank, local)
        return
    if a.workload == "conv":
        run_conv(a, ws, rank, local)
        return
    run_clinical(a, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_clinical(a, ws, rank, local):
    """The headline: TOF list-mode OSEM on the clinical workload. With N ranks every subset's
    events are split into N shards (strong scaling on the same events); each rank runs the fused
    subset step on its shard and the ranks sum their backprojections with one all-reduce per
    subset before the identical update."""
    import numpy as np
    import torch
    from srf_gb300 import _lib, kernels
    from srf_gb300._lib import SRF_RATIO_DIV_NO_NAN
    from srf_gb300.data import Emap, Listmode, Lors
    from srf_gb300.distributed import ShardedOsem, shard_range
    from srf_gb300.geometry import block_full_crystal_table
    from srf_gb300.recon import OsemFullTof

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    _lib.load()
    _lib.set_group_lanes(a.lanes)

    sc, ic, act, lors = make_workload(a, dev, 0)  # every rank draws the same events
    tof = (sc.tof.tof_bin, sc.tof.tof_sigma2)
    n = lors.shape[0]
    n_sub = a.subsets
    stride_b = lors.stride(0) * 4

    # sensitivity image over all crystal pairs (timed apart: first call, then warm best of 3)
    table = torch.as_tensor(block_full_crystal_table(sc), device=dev)
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    emap = kernels.emap_block_full(table, sc.nb_blocks_per_ring, ic.shape, ic.center, ic.size)
    torch.cuda.synchronize()
    emap_cold_s = time.perf_counter() - t0
    emap_warm = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        emap = kernels.emap_block_full(table, sc.nb_blocks_per_ring, ic.shape, ic.center, ic.size)
        e1.record(stream)
        torch.cuda.synchronize()
        emap_warm.append(e0.elapsed_time(e1) / 1000.0)
    del table
    em = kernels.xfast(emap * (1.0 / n_sub))

    # the drop-in's inputs in host memory, in event order (rank 0 times the end-to-end leg)
    host_lors = host_y = None
    h2d_gbps = None
    if not a.no_e2e:
        host_lors = torch.empty(lors.shape, dtype=lors.dtype, pin_memory=True)
        host_lors.copy_(lors)
        host_y = torch.ones(n, dtype=torch.float32, pin_memory=True)
        # raw host-to-device rate of one copy of the LOR array from pinned memory (what the
        # end-to-end leg's copies cost)
        scratch = torch.empty_like(lors)
        scratch.copy_(host_lors, non_blocking=True)
        torch.cuda.synchronize()
        h0, h1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        h0.record(stream)
        scratch.copy_(host_lors, non_blocking=True)
        h1.record(stream)
        torch.cuda.synchronize()
        h2d_gbps = host_lors.numel() * 4 / (h0.elapsed_time(h1) / 1000.0) / 1e9
        del scratch

    # interleaved subsets: subset k is events k, k + n_sub, ... of the list in event order (a
    # strided view, no reordering); this rank keeps its contiguous share of each subset
    n_per = n // n_sub
    n_used = n_per * n_sub
    lo, hi = shard_range(n_per, rank, ws)
    shard_lors = [lors[k:n_used:n_sub][lo:hi] for k in range(n_sub)]
    mine = n_sub * (hi - lo)

    # exact LOR-voxel visits of one iteration (all ranks' events)
    p_fwd = kernels.count_pairs(lors[:n_used], ic.shape, ic.center, ic.size, rules=0, tof=tof, tof_nsigma=a.nsigma)
    p_bwd = kernels.count_pairs(lors[:n_used], ic.shape, ic.center, ic.size, rules=1, tof=tof, tof_nsigma=a.nsigma)
    updates_per_iter = p_fwd + p_bwd

    st = kernels.SubsetState(ic.shape, ic.center, ic.size, dev)
    drv = ShardedOsem(st)

    def iteration(ev=None):
        for k in range(n_sub):
            if ev is not None:
                ev[k][0].record(stream)
            st.subset(shard_lors[k], None, rule=SRF_RATIO_DIV_NO_NAN, eps=1e-5, tof=tof, tof_nsigma=a.nsigma)
            if ev is not None:
                ev[k][1].record(stream)
            drv.reduce()
            st.update(em, guard_zero=True)

    for _ in range(a.warmup):
        iteration()
    torch.cuda.synchronize()

    evs = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)]
            for _ in range(n_sub)] for _ in range(a.steps)]
    clocks = Clocks(local)
    barrier(ws)
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for s_ in range(a.steps):
        iteration(evs[s_])
    stop.record(stream)
    torch.cuda.synchronize()
    barrier(ws)
    clk = clocks.stop()
    ms_total = max_over_ranks(start.elapsed_time(stop), ws, dev)
    ms_step = ms_total / a.steps
    kern_ms = [evs[s_][k][0].elapsed_time(evs[s_][k][1]) for s_ in range(a.steps) for k in range(n_sub)]
    kern_ms_avg = sum(kern_ms) / len(kern_ms)
    value = float(updates_per_iter) / (ms_step / 1000.0)

    # roofline of the dominant kernel (the fused subset step) on this rank's launches. Its binding
    # roof is L2: the gathers (4 B per projector visit) at the best-case L2 load rate plus the
    # reductions (one red.add.f32 per backprojector visit) at the best-case L2 red rate, both
    # measured in this run. Reductions count as load-equivalent bytes at the ratio of the two
    # rates, so achieved / peak = (t_gather + t_red) / launch time.
    share = mine / max(n_used, 1)
    fwd_l = p_fwd * share / n_sub
    bwd_l = p_bwd * share / n_sub
    l2 = l2_peaks(dev)
    t_gather = 4.0 * fwd_l / (l2["read_gbps"] * 1e9)
    t_red = bwd_l / l2["red_per_s"]
    l2_bytes = 4.0 * fwd_l + bwd_l * (l2["read_gbps"] * 1e9 / l2["red_per_s"])
    l2_achieved = l2_bytes / (kern_ms_avg / 1000.0) / 1e9
    hbm_peak, hbm_kind = peaks()
    lor_bytes = (mine / n_sub) * stride_b
    roofline = {"bound": "l2", "achieved": l2_achieved, "peak": l2["read_gbps"], "unit": "GB/s",
                "frac": l2_achieved / l2["read_gbps"],
                "traffic": NCU_TRAFFIC_SUBSET if (mine // n_sub == 2_000_000 and a.nsigma == 3.0) else None,
                "kernel": "k_osem_subset (fused projection+ratio+backprojection)",
                "launch_ms": kern_ms_avg, "t_gather_ms": 1000 * t_gather, "t_red_ms": 1000 * t_red,
                "gather_bytes_per_launch": 4.0 * fwd_l, "red_ops_per_launch": bwd_l,
                "l2_red_peak_per_s": l2["red_per_s"],
                "peak_kind": "measured in this run (srf_calib_l2: L2-resident 32 MB buffer)",
                "achieved_def": "(gather bytes + red ops x read_peak/red_peak) / launch time"}
    roofline_hbm = {"bound": "hbm", "achieved": lor_bytes / (kern_ms_avg / 1000.0) / 1e9,
                    "peak": hbm_peak, "unit": "GB/s",
                    "frac": lor_bytes / (kern_ms_avg / 1000.0) / 1e9 / hbm_peak,
                    "alg_bytes_per_launch": lor_bytes, "peak_kind": hbm_kind,
                    "alg_def": "the launch's LOR rows (28 B each); image and accumulators stay in L2"}

    # FP64 Poisson log-likelihood of the final image over all events:
    # sum_i log(p_i + 1e-5) - sum_j emap_j x_j (p from the projector, emap the full sensitivity)
    llst = kernels.SubsetState(ic.shape, ic.center, ic.size, dev, x0=st.x)
    for k in range(n_sub):
        llst.subset(shard_lors[k], None, rule=SRF_RATIO_DIV_NO_NAN, eps=1e-5, tof=tof,
                    tof_nsigma=a.nsigma, track_loglik=True)
    data_term = sum_over_ranks(float(llst.loglik.item()), ws, dev)
    sens_term = float((emap.double() * st.x.double()).sum().item())
    del llst

    # end to end through the drop-in: OsemFullTof(1 iteration, interleaved subsets) on pinned host
    # LORs and values -- host-to-device copies, the values regrouped by subset, every subset step
    # (with N ranks: this rank's shards and the per-subset all-reduce) -- and the image read back
    # into pinned host memory, every step
    e2e = None
    if host_lors is not None:
        emap_img = Emap(emap, list(ic.center), list(ic.size))
        rec = OsemFullTof(1, n_sub, ic, sc, Listmode(host_y, Lors(host_lors)), emap_img,
                          tof_nsigma=a.nsigma, seed=a.seed, sharded=ws > 1, subsets="interleaved")
        out_host = torch.empty(ic.shape, dtype=torch.float32, pin_memory=True)
        d2h = torch.cuda.Stream(dev)

        def e2e_step():
            # the image read back on a stream of its own, so the next step's kernels do not
            # queue behind it (the allocator keeps the image until the copy is done)
            img = rec()
            ready = torch.cuda.Event()
            ready.record(stream)
            d2h.wait_event(ready)
            with torch.cuda.stream(d2h):
                out_host.copy_(img.data, non_blocking=True)
            img.data.record_stream(d2h)

        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        barrier(ws)
        e_start, e_stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0 = time.perf_counter()
        e_start.record(stream)
        for _ in range(a.steps):
            e2e_step()
        stream.wait_stream(d2h)  # the last image's copy is inside the timed region
        e_stop.record(stream)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - t0) / a.steps
        e_ms = max_over_ranks(max(e_start.elapsed_time(e_stop) / a.steps, 1000 * wall), ws, dev)
        e2e = {"value": float(updates_per_iter) / (e_ms / 1000.0), "unit": UNIT,
               "h2d_bytes_per_step": int(ws * (host_lors.numel() * 4 + host_y.numel() * 4)),
               "d2h_bytes_per_step": int(ws * out_host.numel() * 4), "ms_per_step": e_ms,
               "h2d_gbps_single_copy": h2d_gbps,
               "path": "srf_gb300.OsemFullTof(1 iteration, %d interleaved subsets)() per step on "
                       "pinned host LORs; image copied back" % n_sub}
        del rec
    host_lors = host_y = None

    # CPU baseline on a sample (the oracle, one thread); the GPU subset step on the same sample
    # and image is checked against it
    cpu = parity = None
    if rank == 0 and not a.no_cpu:
        samp = lors[: a.cpu_sample]
        samp_np = samp.cpu().numpy()
        x_np = st.x.contiguous().cpu().numpy()
        threads = 1
        rate, pairs, dt, p_ref, bp_ref = cpu_sample_rate(samp_np, x_np, ic, tof, a.nsigma, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{len(samp_np)} of {n} events: one TOF subset pass (projection, ratio, "
                         f"backprojection) of the oracle, {pairs} visits in {dt:.2f} s"}
        parity = subset_parity(st.x, samp, x_np, p_ref, bp_ref, ic, tof, a.nsigma, dev)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms_step, "s_per_iter": ms_step / 1000.0,
            "higher_is_better": True, "scaling": "strong" if ws > 1 else "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded phantom, events snapped to crystals)",
            "config": dict(workload_config(a), parallelism=f"events sharded over {ws} rank(s), "
                                                           "one all-reduce per subset"),
            "updates_per_iter": updates_per_iter, "pairs_fwd": p_fwd, "pairs_bwd": p_bwd,
            "emap_s": min(emap_warm), "emap_s_first_call": emap_cold_s,
            "emap_lors": int(sc.nb_crystals) ** 2,
            "roofline": roofline, "roofline_hbm": roofline_hbm,
            "parity": parity,
            "loglik_fp64": {"value": data_term - sens_term, "data_term": data_term,
                            "sensitivity_term": sens_term,
                            "def": "sum_i log(p_i + 1e-5) - sum_j emap_j x_j after the timed iterations"},
            "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
            "gpu_launches": a.steps * n_sub * 2,
        }
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
