#!/usr/bin/env python
"""Benchmark: Gterms/s of the shaded visibility DFT + direct-DFT reconstruction.

One step = one vis-DFT pass (K visibilities x J pixels, geometric Moon
occlusion inline) followed by one reconstruction pass over the same K x J
terms: 2*K*J terms.  Workload: 10 MHz, 8 satellites on a 30 deg inclined
300 km lunar orbit, 28 baselines x 65,536 snapshots = 1,835,008 float32 uvw,
196,608 Fibonacci-sphere pixels (power-law diffuse sky + 500 point sources),
synthetic and seeded.  Inputs (~40 MB) are smaller than L2, so L2 is flushed
(a 256 MB write) before every timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU restatement (the FP64
oracle, all host threads) on a bounded sample per step; where the reference's
own CUDA kernels were built from its sources (oracle/_ref) it also times the
reference's plain kernels (visscal + imagerecon of vissGen10M_shade) on the GPU.
"""
from __future__ import annotations

import argparse
import csv
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gterms/s shaded vis-DFT + recon, 1 GB300, chosen vs plain at ≤1e-5 rel err"
# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from one ncu
# capture of this workload at full size (the command is kept with the ncu summaries).
TRAFFIC_BYTES = {"cfg2_10MHz": {"vis_fast_kernel": 198.76e6, "recon_fast_kernel": 297.08e6}}
UNIT = "Gterms/s"
L2_FLUSH_BYTES = 256 << 20


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="cfg2_10MHz")
    ap.add_argument("--precision", choices=["auto", "fast", "comp"], default="auto")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-ref-cuda", action="store_true")
    ap.add_argument("--no-stage1", action="store_true", help="skip the stage-1 (uvw generation) record")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched 64-channel record")
    ap.add_argument("--no-largest", action="store_true", help="skip the 30 MHz (largest configuration) record")
    ap.add_argument("--mask", choices=["geometric", "none"], default="geometric",
                    help="occlusion mask of the DFT passes (none: every term computed, for profiling)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target CPU work of the baseline sample")
    return ap.parse_args()


# ------------------------------------------------------------------ distributed
def dist_setup(group: bool = True, cuda: bool = True):
    """(world size, rank, local rank) from the launcher's environment; with `group`
    a NCCL process group over the ranks (N > 1), with `cuda` this rank's GPU selected."""
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if not group:
        if cuda:
            torch.cuda.set_device(local)
        return ws, rank, local
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    """The slowest rank's time (replicas: each rank runs the whole workload on its GPU)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region (the body of
    the `with`).  nvidia-smi is started and its first sample awaited before the body
    runs: its start-up stalls the GPU for a few hundred ms, which must not fall inside a
    short timed region.  Samples are time-stamped and those around the body kept."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
            deadline = time.time() + 10.0
            while time.time() < deadline and self.proc.poll() is None:
                with open(self.path) as f:
                    if f.read().count("\n") >= 2:
                        break
                time.sleep(0.02)
        except Exception:
            self.proc = None
        self.t0 = time.time()
        return self

    def __exit__(self, *a):
        self.t1 = time.time()
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def _in_window(self, stamp: str) -> bool:
        import datetime
        try:
            t = datetime.datetime.strptime(stamp.strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return True
        return self.t0 - 0.3 <= t <= self.t1 + 0.3

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        rows = []
        with open(self.path) as f:
            for r in csv.reader(f):
                if len(r) >= 10:
                    rows.append([x.strip() for x in r])
        os.unlink(self.path)
        window = [r for r in rows if self._in_window(r[0])]
        rows = [r[1:] for r in (window or rows)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows if r[3].replace(".", "").isdigit()), default=None)}


# ------------------------------------------------------------------ workload
def load_workload(name, device="cuda"):
    import torch
    from viss_recon_shade_gb300.synth import WORKLOADS, make_sky, make_uvw
    wl = WORKLOADS[name]
    d = make_uvw(wl, device=device)
    l, m, n, b = make_sky(wl)
    t = lambda a: torch.from_numpy(a).to(device)  # noqa: E731
    d.update(l=t(l), m=t(m), n=t(n), b=t(b))
    torch.cuda.synchronize()
    return wl, d


def precision_name(d, pref) -> str:
    """'fast' or 'compensated' for this workload's uvw (tensors or arrays)."""
    if pref == "fast":
        return "fast"
    if pref == "comp":
        return "compensated"
    umax = max(float(abs(d[k]).max()) for k in ("u", "v", "w"))
    # the fast path's phase error grows as |uvw| * 2^-33 turns per coordinate; up to
    # |uvw| ~ 1.2e4 (30 MHz, 100 km baselines) it measures <= 1e-5 against FP64
    # (tests/test_gpu_precision.py), beyond that the compensated path is needed
    return "fast" if umax <= 12000 else "compensated"


def choose_precision(d, pref):
    import viss_recon_shade_gb300 as V
    return {"fast": V.PREC_FAST, "compensated": V.PREC_COMPENSATED}[precision_name(d, pref)]


def workload_config(wl, K, J, precision, ws, mask="geometric"):
    """The `config` of both arms' lines (same workload, same keys and values)."""
    return {"workload": wl.name, "K": K, "J": J, "terms_per_step": int(2 * K * J), "snapshots": wl.snapshots,
            "baselines": wl.npairs, "freq_hz": wl.freq_hz, "mask": mask, "precision": precision,
            "l2": "flushed (256 MB write) before each timed step", "parallelism": f"replicas x{ws}"}


def run_ours(args, ws, rank, local):
    import torch
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300 import _lib as L
    wl, d = load_workload(args.workload)
    K, J = d["u"].numel(), d["l"].numel()
    prec = choose_precision(d, args.precision)
    cfg = V.DftConfig.geometric(precision=prec, occluded_value=0.0)
    if args.mask == "none":
        cfg = cfg.with_(mask=V.MASK_NONE, recon_mask=V.RECON_MASK_NONE)
    geo = dict(snap=d["snap"], pair=d["pair"], sat_pos=d["sat_pos"])
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    Vout = torch.empty(K, dtype=torch.complex64, device="cuda")
    Fout = torch.empty(J, dtype=torch.complex64, device="cuda")

    def step():
        V.vis_dft(cfg, d["u"], d["v"], d["w"], d["l"], d["m"], d["n"], d["b"], out=Vout, **geo)
        V.recon(cfg, d["u"], d["v"], d["w"], Vout, d["l"], d["m"], d["n"], out=Fout, **geo)

    # warm-up steps run exactly what a timed step runs, the L2 flush included: the first
    # use of a library kernel on a fresh machine may JIT it (torch's fill kernel for
    # this GPU, cached afterwards), which must not land in the timed region
    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = L.lib.viss_launch_count()
    with ClockSampler(local) as clk:
        barrier(ws)
        torch.cuda.synchronize()
        t0e.record(st)
        for i in range(args.steps):
            flush.zero_()  # L2 flush between timed steps
            ev[i][0].record(st)
            V.vis_dft(cfg, d["u"], d["v"], d["w"], d["l"], d["m"], d["n"], d["b"], out=Vout, **geo)
            ev[i][1].record(st)
            V.recon(cfg, d["u"], d["v"], d["w"], Vout, d["l"], d["m"], d["n"], out=Fout, **geo)
            ev[i][2].record(st)
        t1e.record(st)
        torch.cuda.synchronize()
        barrier(ws)
    launches = int(L.lib.viss_launch_count() - n0)
    total_ms = max_over_ranks(t0e.elapsed_time(t1e), ws)
    vis_ms = statistics.mean(e[0].elapsed_time(e[1]) for e in ev)
    rec_ms = statistics.mean(e[1].elapsed_time(e[2]) for e in ev)
    terms_step = 2.0 * K * J
    value = terms_step * args.steps * ws / (total_ms * 1e-3) / 1e9

    # ---- e2e through the public API with host buffers ----------------------
    host = {k: d[k].cpu().pin_memory() for k in ("u", "v", "w", "snap", "pair", "l", "m", "n", "b", "sat_pos")}
    dev = {k: torch.empty_like(d[k]) for k in host}
    hV = torch.empty(K, dtype=torch.complex64).pin_memory()
    hF = torch.empty(J, dtype=torch.complex64).pin_memory()
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    d2h = hV.numel() * 8 + hF.numel() * 8

    def e2e_step():
        for k in host:
            dev[k].copy_(host[k], non_blocking=True)
        g = dict(snap=dev["snap"], pair=dev["pair"], sat_pos=dev["sat_pos"])
        Vd = V.vis_dft(cfg, dev["u"], dev["v"], dev["w"], dev["l"], dev["m"], dev["n"], dev["b"], **g)
        Fd = V.recon(cfg, dev["u"], dev["v"], dev["w"], Vd, dev["l"], dev["m"], dev["n"], **g)
        hV.copy_(Vd, non_blocking=True)
        hF.copy_(Fd, non_blocking=True)

    e2e_step()
    torch.cuda.synchronize()
    barrier(ws)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2e_steps = max(2, min(args.steps, 5))
    e0.record(st)
    for _ in range(e2e_steps):
        flush.zero_()
        e2e_step()
    e1.record(st)
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1), ws)
    e2e_value = terms_step * e2e_steps * ws / (e2e_ms * 1e-3) / 1e9

    # ---- roofline: SFU pipe (2 SFU ops per term) ------------------------------
    import ctypes as C
    probe_out = torch.zeros(4, device="cuda")
    ops = C.c_int64(0)
    for _ in range(2):
        L.check(L.lib.viss_sfu_probe(4096, 8, C.c_void_p(probe_out.data_ptr()), C.byref(ops),
                                     C.c_void_p(st.cuda_stream)), "probe")
    pe0, pe1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    pe0.record(st)
    L.check(L.lib.viss_sfu_probe(4096, 8, C.c_void_p(probe_out.data_ptr()), C.byref(ops),
                                 C.c_void_p(st.cuda_stream)), "probe")
    pe1.record(st)
    torch.cuda.synchronize()
    sfu_peak = ops.value / (pe0.elapsed_time(pe1) * 1e-3) / 1e9  # G SFU ops / s
    dom_ms, dom = (vis_ms, "vis_fast_kernel") if vis_ms >= rec_ms else (rec_ms, "recon_fast_kernel")
    achieved = 2.0 * K * J / (dom_ms * 1e-3) / 1e9
    props = torch.cuda.get_device_properties(0)
    traffic = TRAFFIC_BYTES.get(wl.name, {}).get(dom)
    hbm_peak, hbm_src = 6800.0, "fallback 6.8 TB/s"
    try:
        hbm_peak = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
        hbm_src = "MEASURED_PEAKS.json hbm_gbs (measured copy bandwidth)"
    except Exception:
        pass
    hbm = None
    if traffic:
        gbs = traffic / (dom_ms * 1e-3) / 1e9
        hbm = {"achieved": round(gbs, 2), "peak": hbm_peak, "unit": "GB/s", "frac": round(gbs / hbm_peak, 5),
               "peak_source": hbm_src}
    # the path is bound by the SFU (sin, cos per term), not by HBM or the tensor cores
    roofline = {"bound": "sfu", "kernel": dom, "achieved": round(achieved, 2), "peak": round(sfu_peak, 2),
                "unit": "G SFU op/s", "frac": round(achieved / sfu_peak, 4),
                "peak_source": "measured: viss_sfu_probe (8 independent __sincosf chains per thread) in this run",
                "algorithmic_per_term": "2 SFU ops (sin, cos) + 6 FMA-pipe ops (vis) / 8 (recon)",
                "traffic": traffic, "traffic_unit": "bytes per launch (ncu)", "hbm": hbm,
                "sm_count": props.multi_processor_count,
                "vis_ms": round(vis_ms, 3), "recon_ms": round(rec_ms, 3)}

    # ---- plain (the reference's FP32 method restated) -------------------------
    plain = None
    if not args.no_plain:
        pcfg = cfg.with_(precision=V.PREC_PLAIN)
        V.vis_dft(pcfg, d["u"], d["v"], d["w"], d["l"], d["m"], d["n"], d["b"], out=Vout, **geo)
        V.recon(pcfg, d["u"], d["v"], d["w"], Vout, d["l"], d["m"], d["n"], out=Fout, **geo)  # warm-up
        torch.cuda.synchronize()
        p0, p1, p2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        flush.zero_()
        p0.record(st)
        V.vis_dft(pcfg, d["u"], d["v"], d["w"], d["l"], d["m"], d["n"], d["b"], out=Vout, **geo)
        p1.record(st)
        V.recon(pcfg, d["u"], d["v"], d["w"], Vout, d["l"], d["m"], d["n"], out=Fout, **geo)
        p2.record(st)
        torch.cuda.synchronize()
        pms = p0.elapsed_time(p2)
        plain = {"value": round(terms_step / (pms * 1e-3) / 1e9, 3), "unit": UNIT,
                 "vis_ms": round(p0.elapsed_time(p1), 2), "recon_ms": round(p1.elapsed_time(p2), 2),
                 "what": "PREC_PLAIN: the reference's FP32 phase (u*l/d + ...), precise sincosf, "
                         "one thread per visibility / pixel, same masks"}
        step()  # restore the chosen outputs
        torch.cuda.synchronize()

    # ---- the reference programs' own mask on the same inputs ------------------
    # REF_QUIRK windows (RES 20940, the shade10M grid) from viss_shade_windows on these
    # uvw, the reference's phase convention and occluded value: the inputs the
    # reference arm's ref_cuda_* legs give the reference's kernels
    ref_mode = None
    if not args.no_ref_cuda and ws == 1:
        RES = 20940
        raw, _ = V.shade_windows(d["u"], d["v"], d["w"], RES)
        shade = V.normalise_shade(raw)
        rcfg = V.DftConfig.reference(RES, precision=prec)
        Vr, Fr = torch.empty_like(Vout), torch.empty_like(Fout)
        r = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        for i in range(2):  # a warm-up pass, then the timed one
            flush.zero_()
            r[0].record(st)
            V.vis_dft(rcfg, d["u"], d["v"], d["w"], d["l"], d["m"], d["n"], d["b"], shade=shade, out=Vr)
            r[1].record(st)
            V.recon(rcfg, d["u"], d["v"], d["w"], Vr, d["l"], d["m"], d["n"], shade=shade, out=Fr)
            r[2].record(st)
            torch.cuda.synchronize()
        rms = r[0].elapsed_time(r[2])
        ref_mode = {"value": round(terms_step / (rms * 1e-3) / 1e9, 3), "unit": UNIT,
                    "vis_ms": round(r[0].elapsed_time(r[1]), 2), "recon_ms": round(r[1].elapsed_time(r[2]), 2),
                    "precision": precision_name(d, args.precision),
                    "what": "REF_QUIRK: the reference programs' window mask as written (vissGen10M_shade.cu:130), "
                            "windows from viss_shade_windows at RES 20940 on these uvw (bit-exact with the "
                            "reference's stage 2), its phase convention and occluded value 240: the inputs of "
                            "the reference arm's ref_cuda_* legs"}
        del Vr, Fr, shade, raw

    # ---- CPU baseline (oracle, bounded sample) + accuracy on the sample -------
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args, wl, d, Vout, Fout, cfg)

    line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (fixed-point i32 phase)",
            "data": "synthetic (seeded orbit + Fibonacci sky)",
            "config": workload_config(wl, K, J, precision_name(d, args.precision), ws, args.mask),
            "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": e2e_steps},
            "roofline": roofline, "gpu_launches": launches, "clocks": clk.summary(),
            "plain": plain, "cpu_baseline": cpu}
    if ref_mode:
        line["ref_mode"] = ref_mode
    if plain:
        line["speedup_vs_plain"] = round(value / plain["value"], 2)
    if not args.no_stage1:
        # stage 1 of the path (positions -> unique uvw) at the reference's own size, for
        # the record; `--workload stage1` reports it in full
        del Vout, Fout, flush
        torch.cuda.empty_cache()
        K1, n1, ms1, (_, uu, vv, ww) = stage1_passes(3, 3)
        line["stage1"] = {"value": round(K1 / (sum(ms1) * 1e-3) / 1e9, 3), "unit": "G uvw rows/s",
                          "ms_per_pass": round(sum(ms1), 2), "uvw_rows": K1, "unique_rows": n1,
                          "stage_ms": {"positions": round(ms1[0], 2), "unique_fused": round(ms1[1], 2)},
                          "what": "MIncline_generate_uvw_float at its own size (8 satellites, 864,000 samples "
                                  "an orbit, 140 orbits, 10 MHz): positions + viss_unique_uvw"}
        if not args.no_ref_cuda:
            line["stage1"]["reference"], line["stage2"] = reference_stages(uu, vv, ww, K1)
        del uu, vv, ww
        torch.cuda.empty_cache()
    if not args.no_batch and ws == 1:
        # the batched multi-channel configuration (64 channels, one persistent graph-replayed
        # launch per pass); `--workload batch64` reports it as its own line
        if "Vout" in locals():
            del Vout, Fout, flush
            torch.cuda.empty_cache()
        b = batch_record("batch64", 3, 2, args.precision, sfu_peak=sfu_peak)
        line["batch64"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "vis_ms", "recon_ms", "roofline",
                                             "plain_per_channel", "speedup_vs_plain", "accuracy", "clocks",
                                             "gpu_launches_per_step")}
        line["batch64"]["config"] = {k: b["config"][k] for k in ("workload", "channels", "K", "J", "terms_per_step",
                                                                  "launch")}
        line["batch64"]["autotune_best"] = b["autotune"]["best"]
        torch.cuda.empty_cache()
    if not args.no_largest and ws == 1 and args.workload != "cfg5_30MHz":
        if "Vout" in locals():
            del Vout, Fout, flush
            torch.cuda.empty_cache()
        line["cfg5"] = largest_record(args.precision, sfu_peak, local)
        torch.cuda.empty_cache()
    if rank == 0:
        print(json.dumps(line), flush=True)


def largest_record(precision, sfu_peak, local, steps=2, warmup=1):
    """The largest configuration (30 MHz, 16 satellites: 7,864,320 visibilities x
    786,432 pixels, 1.24e13 terms per step, geometric mask) through the same public
    calls as the headline: one warm-up step, then `steps` timed ones (CUDA events; its
    inputs are far larger than L2)."""
    import torch
    import viss_recon_shade_gb300 as V
    wl, d = load_workload("cfg5_30MHz")
    K, J = d["u"].numel(), d["l"].numel()
    prec = choose_precision(d, precision)
    cfg = V.DftConfig.geometric(precision=prec, occluded_value=0.0)
    geo = dict(snap=d["snap"], pair=d["pair"], sat_pos=d["sat_pos"])
    Vout = torch.empty(K, dtype=torch.complex64, device="cuda")
    Fout = torch.empty(J, dtype=torch.complex64, device="cuda")
    st = torch.cuda.current_stream()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(warmup + steps)]
    with ClockSampler(local) as clk:
        for e in ev:
            e[0].record(st)
            V.vis_dft(cfg, d["u"], d["v"], d["w"], d["l"], d["m"], d["n"], d["b"], out=Vout, **geo)
            e[1].record(st)
            V.recon(cfg, d["u"], d["v"], d["w"], Vout, d["l"], d["m"], d["n"], out=Fout, **geo)
            e[2].record(st)
        torch.cuda.synchronize()
    timed = ev[warmup:]
    vis_ms = statistics.mean(e[0].elapsed_time(e[1]) for e in timed)
    rec_ms = statistics.mean(e[1].elapsed_time(e[2]) for e in timed)
    terms = 2.0 * K * J
    rec = {"value": round(terms / ((vis_ms + rec_ms) * 1e-3) / 1e9, 3), "unit": UNIT,
           "ms_per_step": round(vis_ms + rec_ms, 2), "vis_ms": round(vis_ms, 2), "recon_ms": round(rec_ms, 2),
           "steps": steps, "warmup": warmup, "clocks": clk.summary(),
           "config": workload_config(wl, K, J, precision_name(d, precision), 1)}
    rec["config"]["l2"] = "inputs far larger than L2 (no flush)"
    if sfu_peak:
        dom_ms, dom = (vis_ms, "vis_fast_kernel") if vis_ms >= rec_ms else (rec_ms, "recon_fast_kernel")
        achieved = terms / (dom_ms * 1e-3) / 1e9
        rec["roofline"] = {"bound": "sfu", "kernel": dom, "achieved": round(achieved, 2), "peak": round(sfu_peak, 2),
                           "unit": "G SFU op/s", "frac": round(achieved / sfu_peak, 4),
                           "peak_source": "measured: viss_sfu_probe in this run"}
    del Vout, Fout, d
    return rec


def reference_stages(uu, vv, ww, K1, RES=20940):
    """The reference's own stage 1 and stage 2 on the same GPU, beside ours.
    Stage 1 (MIncline_generate_uvw_float.cu:215-397 at its size): its orbit, window and
    computeUVW kernels from its sources, per ordered pair thrust::sort + unique with its
    comparators (restated, oracle/ref_thrust.cu), the concatenation and the global
    sort + unique -- compared row for row (bitwise) with ours (uu, vv, ww).  Stage 2
    (shade10M.cu:188-224, RES 20940) on those unique rows: its Cart2SphKernel, its FP32
    thrust mean radius (restated; it copies r into a device_vector first, as the
    reference's r is one) and ShadeMatrix, against viss_shade_windows on the same rows."""
    import torch
    try:
        import viss_recon_shade_gb300 as V
        from oracle import ref_cuda, ref_thrust
        from viss_recon_shade_gb300.synth import REF_R1, REF_R2
        if not ref_cuda.available():
            return {"unavailable": "reference kernels not built (oracle/_ref missing)"}, None
        cfg = V.OrbitConfig()
        ref_cuda.mincline_unique(8, 8640, 2, 1, 1e7, REF_R1, REF_R2)  # module loads, first launches
        rows, ms = ref_cuda.mincline_unique(cfg.nsat, cfg.orbit_res, cfg.orbit_counts, 1, 1e7, REF_R1, REF_R2,
                                            timed=True)
        ours = torch.stack([uu, vv, ww], 1)
        same1 = rows.shape == ours.shape and torch.equal(rows.view(torch.int32), ours.view(torch.int32))
        s1 = {"value": round(K1 / (ms["total"] * 1e-3) / 1e9, 3), "unit": "G uvw rows/s",
              "ms_per_pass": round(ms["total"], 1),
              "stage_ms": {k: round(v, 1) for k, v in ms.items() if k != "total"}, "unique_rows": int(rows.shape[0]),
              "identical_rows": bool(same1),
              "what": "the reference's calculateOrbit / uvwPosition / computeUVW kernels (its sources) + per-pair "
                      "thrust sort/unique with its comparators + global sort/unique (thrust, restated)"}
        del rows
        u, v, w = (x.contiguous() for x in (uu, vv, ww))
        st = torch.cuda.current_stream()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ref_cuda.shade_windows(u[:4096], v[:4096], w[:4096], RES, 3000.0)  # warm
        V.shade_windows(u, v, w, RES)
        torch.cuda.synchronize()
        ev[0].record(st)
        _, mean_r = ref_thrust.mean_r(ref_cuda.cart2sph_r(u, v, w))
        ref_win, _ = ref_cuda.shade_windows(u, v, w, RES, mean_r)
        ev[1].record(st)
        win, m_ours = V.shade_windows(u, v, w, RES)
        ev[2].record(st)
        torch.cuda.synchronize()
        ref_ms, our_ms = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
        n = u.numel()
        s2 = {"value": round(n / (our_ms * 1e-3) / 1e9, 2), "unit": "G rows/s", "rows": n, "res": RES,
              "ms": round(our_ms, 3),
              "reference": {"value": round(n / (ref_ms * 1e-3) / 1e9, 2), "unit": "G rows/s", "ms": round(ref_ms, 3)},
              "identical_windows": bool(torch.equal(ref_win, win)), "mean_r_equal": bool(float(m_ours) == mean_r),
              "what": "shade windows of the stage-1 rows: Cart2Sph + FP32 mean radius + ShadeMatrix"}
        return s1, s2
    except Exception as e:  # reported, not fatal
        return {"unavailable": f"{type(e).__name__}: {e}"}, None


def cpu_baseline(args, wl, d, Vout, Fout, cfg):
    """FP64 oracle (the reference formulas restated, OpenMP) on a bounded sample of
    the workload: `nr` visibility rows x all pixels plus `np_` pixels x all
    visibilities.  Also reports the GPU's error on exactly those rows/pixels."""
    import numpy as np
    from oracle import oracle as O
    O.build()
    h = lambda t: t.cpu().numpy()  # noqa: E731
    u, v, w, snap, pair, pos = (h(d[k]) for k in ("u", "v", "w", "snap", "pair", "sat_pos"))
    l, m, n, b = (h(d[k]) for k in ("l", "m", "n", "b"))
    K, J = u.size, l.size
    thr = O.max_threads()
    ocfg = O.make_cfg(mask_mode=O.MASK_GEOMETRIC if args.mask == "geometric" else O.MASK_NONE,
                      phase_scale=cfg.phase_scale, n_offset=cfg.n_offset,
                      occluded_value=cfg.occluded_value, norm=1.0 / K)
    # calibrate, then size the sample to ~cpu_seconds
    rows = np.arange(0, K, max(1, K // 64))[:64]
    t0 = time.perf_counter()
    geo_s = O.make_geo(pos, snap[rows], pair[rows])
    O.vis_dft(ocfg, u[rows], v[rows], w[rows], l, m, n, b, geo=geo_s, nthreads=thr)
    rate = rows.size * J / (time.perf_counter() - t0)
    target_terms = rate * args.cpu_seconds
    whole = lambda x, cap: int(min(cap, max(thr, round(x / thr) * thr)))  # noqa: E731  (equal shares a thread)
    nr = whole(target_terms / 2 / J, K)
    np_ = whole(target_terms / 2 / K, J)
    ridx = np.linspace(0, K - 1, nr).astype(np.int64)
    pidx = np.linspace(0, J - 1, np_).astype(np.int64)
    t0 = time.perf_counter()
    geo_r = O.make_geo(pos, snap[ridx], pair[ridx])
    Vo = O.vis_dft(ocfg, u[ridx], v[ridx], w[ridx], l, m, n, b, geo=geo_r, nthreads=thr)
    geo_all = O.make_geo(pos, snap, pair)
    Vg = h(Vout)
    Fo = O.recon(ocfg, u, v, w, None, Vg, l[pidx], m[pidx], n[pidx], geo=geo_all, nthreads=thr)
    dt = time.perf_counter() - t0
    terms = nr * J + np_ * K
    Fg = h(Fout)[pidx]
    ev = np.linalg.norm(Vg[ridx] - Vo) / np.linalg.norm(Vo)
    ef = np.linalg.norm(Fg - Fo) / np.linalg.norm(Fo)
    evm = np.abs(Vg[ridx] - Vo).max() / np.abs(Vo).max()
    efm = np.abs(Fg - Fo).max() / np.abs(Fo).max()
    return {"value": round(terms / dt / 1e9, 4), "unit": UNIT, "cores": thr, "kind": "port",
            "sample": f"FP64 oracle: {nr} visibilities x {J} pixels + {np_} pixels x {K} visibilities "
                      f"({terms:.3g} terms, {dt:.1f} s)",
            "gpu_rel_err_on_sample": {"vis_rms": float(ev), "vis_max": float(evm), "recon_rms": float(ef),
                                      "recon_max": float(efm),
                                      "definitions": {"rms": "||gpu - fp64|| / ||fp64|| over the sample",
                                                      "max": "max |gpu - fp64| / max |fp64| over the sample"}}}


# ------------------------------------------------------------------ reference arm
def _synth_standalone():
    """synth.py loaded by path: the reference arm must not load the product library
    (importing the package would)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("viss_synth_standalone",
                                                  ROOT / "viss_recon_shade_gb300" / "synth.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[spec.name] = mod  # dataclasses look their module up
    spec.loader.exec_module(mod)
    return mod


def reference_workload(name):
    """The workload's inputs built on the host without the product: satellite
    positions and continuous uvw from the oracle's FP64 restatement of calculateOrbit /
    uvwPosition / computeUVW, the sky from numpy.  Same shapes and generators as the
    product arm's (the last bits of a few uvw may differ: host vs device FP64 sin/cos)."""
    import numpy as np
    from oracle import oracle as O
    S = _synth_standalone()
    wl = S.WORKLOADS[name]
    r1, r2 = S.log_separations(wl.nsat)
    oc = O.make_orbit_cfg(wl.nsat, wl.orbit_res, wl.orbit_counts, index=1, a_km=wl.a_km, incl_deg=wl.incl_deg,
                          r1_m=r1, r2_m=r2)
    pos64 = O.orbit_positions_f64(oc, nthreads=O.max_threads())
    u, v, w = O.uvw_f64(pos64, wl.lambda_m, ordered=wl.ordered)
    pairs = [(a, b) for a in range(wl.nsat) for b in range(wl.nsat) if (a != b if wl.ordered else a < b)]
    packed = np.array([a | (b << 16) for a, b in pairs], np.int32)
    snap = np.repeat(np.arange(pos64.shape[0], dtype=np.int32), len(pairs))
    pair = np.tile(packed, pos64.shape[0])
    l, m, n, b = S.make_sky(wl)
    return wl, dict(u=u, v=v, w=w, snap=snap, pair=pair, sat_pos=pos64.astype(np.float32), l=l, m=m, n=n, b=b)


def run_reference(args, ws, rank, local):
    """The reference's CPU implementation of the path (the FP64 restatement of
    visscal / imagerecon, oracle/viss_oracle.cpp, every host thread) on a bounded
    sample of the same workload per step: nr visibilities x all J pixels (vis) and
    np_ pixels x all K visibilities (recon), both multiples of the thread count so
    that every thread gets the same share.  Where the reference's own kernels were
    built from its sources (oracle/_ref), their full-size GPU timings are added as
    ref_cuda_* keys.  Nothing here loads the product library."""
    if rank != 0:
        return
    import numpy as np
    from oracle import oracle as O
    O.build()
    wl, d = reference_workload(args.workload)
    u, v, w, snap, pair, pos = (d[k] for k in ("u", "v", "w", "snap", "pair", "sat_pos"))
    l, m, n, b = (d[k] for k in ("l", "m", "n", "b"))
    K, J = u.size, l.size
    thr = O.max_threads()
    ocfg = O.make_cfg(mask_mode=O.MASK_GEOMETRIC if args.mask == "geometric" else O.MASK_NONE, phase_scale=1.0,
                      n_offset=-1.0, occluded_value=0.0, norm=1.0 / K)
    geo_all = O.make_geo(pos, snap, pair)
    # calibrate on 4 rows a thread, then size the sample to ~cpu_seconds / 4 per step
    rows = np.linspace(0, K - 1, 4 * thr).astype(np.int64)
    t0 = time.perf_counter()
    O.vis_dft(ocfg, u[rows], v[rows], w[rows], l, m, n, b, geo=O.make_geo(pos, snap[rows], pair[rows]), nthreads=thr)
    rate = rows.size * J / (time.perf_counter() - t0)
    tgt = rate * args.cpu_seconds / 4.0
    whole = lambda x, cap: int(min(cap, max(thr, round(x / thr) * thr)))  # noqa: E731
    nr = whole(tgt / 2 / J, K)
    np_ = whole(tgt / 2 / K, J)
    ridx = np.linspace(0, K - 1, nr).astype(np.int64)
    pidx = np.linspace(0, J - 1, np_).astype(np.int64)
    geo_r = O.make_geo(pos, snap[ridx], pair[ridx])
    Vs = np.zeros(K, np.complex64)

    def step():
        Vo = O.vis_dft(ocfg, u[ridx], v[ridx], w[ridx], l, m, n, b, geo=geo_r, nthreads=thr)
        Vs[ridx] = Vo
        O.recon(ocfg, u, v, w, None, Vs, l[pidx], m[pidx], n[pidx], geo=geo_all, nthreads=thr)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = time.perf_counter() - t0
    terms = (nr * J + np_ * K) * args.steps
    value = terms / dt / 1e9
    line = {"metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded orbit + Fibonacci sky)",
            "impl": "reference",
            "config": workload_config(wl, K, J, precision_name(d, args.precision), ws, args.mask),
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": thr, "kind": "port",
                             "sample": f"per step {nr} visibilities x {J} pixels + {np_} pixels x {K} visibilities "
                                       f"({nr * J + np_ * K:.3g} terms), FP64 restatement of visscal/imagerecon "
                                       f"(oracle/viss_oracle.cpp) with the {args.mask} mask, OpenMP on every host "
                                       "thread"},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_ref_cuda:
        line["ref_cuda_plain"] = ref_cuda_plain(wl, d)
        # the reference's own rewrites of the same kernels, for context
        line["ref_cuda_optim1"] = ref_cuda_plain(wl, d, "vissGen10M_shade_optim1")
        line["ref_cuda_optim2"] = ref_cuda_plain(wl, d, "vissGen10M_shade_optim2")
    print(json.dumps(line), flush=True)


def reference_windows(u, v, w, RES):
    """Normalised REF windows [K, 4] (CUDA int32) from the reference's own stage 2:
    its Cart2SphKernel and ShadeMatrix (oracle/ref_cuda.py), its thrust mean radius
    restated (oracle/ref_thrust.cu), then the normalisation on load
    (vissGen10M_shade.cu:383-399)."""
    import torch
    from oracle import ref_cuda, ref_thrust
    _, mean_r = ref_thrust.mean_r(ref_cuda.cart2sph_r(u, v, w))
    raw, _ = ref_cuda.shade_windows(u, v, w, RES, mean_r)
    t, p = raw[:, :2], raw[:, 2:]
    return torch.stack([t.min(1).values - 1, t.max(1).values - 1, p.min(1).values - 1, p.max(1).values - 1], 1)


def ref_cuda_plain(wl, d, variant="vissGen10M_shade"):
    """The reference's own kernels (visscal + imagerecon of `variant`: vissGen10M_shade,
    or its _optim1 / _optim2 rewrites; compiled from its sources into oracle/_ref) on
    the full workload, with its REF window mask (RES 20940) from its own stage 2."""
    try:
        import torch
        from oracle import ref_cuda
        if not ref_cuda.available():
            return {"unavailable": "reference kernels not built (oracle/_ref missing)"}
        t = {k: torch.from_numpy(d[k]).cuda() for k in ("u", "v", "w", "l", "m", "n", "b")}
        K, J = t["u"].numel(), t["l"].numel()
        RES = 20940
        Ms = [x.contiguous() for x in reference_windows(t["u"], t["v"], t["w"], RES).unbind(1)]
        FF = t["b"]
        nxq = torch.arange(J, dtype=torch.float32, device="cuda")
        cl = torch.ones(J, dtype=torch.int32, device="cuda")
        wgt = torch.ones(K, dtype=torch.float32, device="cuda")
        nclip = t["n"].clamp(-1, 1)
        args = (t["u"], t["v"], t["w"], t["l"], t["m"], nclip)
        st = torch.cuda.current_stream()
        # warm both kernels on a slice (module load, first launch)
        v0 = ref_cuda.visscal(variant, 8192, J, RES, FF, *args, *[x[:8192] for x in Ms], nxq, cl)
        ref_cuda.imagerecon(variant, 8192, J, RES, v0, *(x[:8192] if x.numel() == K else x for x in args),
                            wgt[:8192], *[x[:8192] for x in Ms])
        torch.cuda.synchronize()
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(st)
        viss = ref_cuda.visscal(variant, K, J, RES, FF, *args, *Ms, nxq, cl)
        e1.record(st)
        ref_cuda.imagerecon(variant, K, J, RES, viss, *args, wgt, *Ms)
        e2.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e2)
        return {"value": round(2.0 * K * J / (ms * 1e-3) / 1e9, 3), "unit": UNIT,
                "vis_ms": round(e0.elapsed_time(e1), 1), "recon_ms": round(e1.elapsed_time(e2), 1),
                "what": f"reference {variant} visscal + imagerecon, unmodified device code, "
                        "REF window mask from the reference's own shade windows, one pass"}
    except Exception as e:  # reported, not fatal: the CPU line above is the reference arm
        return {"unavailable": f"{type(e).__name__}: {e}"}


# ------------------------------------------------------------------ batched channels
def run_batch(args, ws, rank, local):
    """--workload batch64: the batched-channel line (batch_record)."""
    line = batch_record(args.workload, args.steps, args.warmup, args.precision, ws, local)
    if rank == 0:
        print(json.dumps(line), flush=True)


def batch_record(workload, steps, warmup, precision, ws=1, local=0, sfu_peak=None):
    """64 channels log-spaced over 1-30 MHz, 28 baselines x U[4096, 65536] snapshots
    each, 49,152 pixels with per-channel power-law brightness, geometric mask; one
    persistent vis launch + one persistent recon launch per step, replayed from a
    CUDA graph, launch parameters from the autotuner (timed on every 8th channel).
    Compared with the reference's form: per-channel plain launches, timed on 4
    channels spread over the band.  With sfu_peak (G SFU op/s) the dominant pass's
    roofline fraction is added."""
    import numpy as np
    import torch
    import viss_recon_shade_gb300 as V
    from viss_recon_shade_gb300 import _lib as L
    from viss_recon_shade_gb300.synth import BATCH_WORKLOADS, make_batch
    bw = BATCH_WORKLOADS[workload]
    d = make_batch(bw)
    t = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    lg, mg, ng = t(d["l"]), t(d["m"]), t(d["n"])
    prec = choose_precision(d, precision)
    cfg = V.DftConfig.geometric(precision=prec, occluded_value=0.0)
    ro = d["row_off"]
    K, J, nch = int(ro[-1]), bw.J, bw.nch

    def make(chans, c=cfg):
        r = np.concatenate([[0], np.cumsum([ro[i + 1] - ro[i] for i in chans])]).astype(np.int64)
        if list(chans) == list(range(nch)):
            sel = slice(None)
            bright = d["bright"]
        else:
            idx = torch.cat([torch.arange(int(ro[i]), int(ro[i + 1]), device="cuda") for i in chans])
            sel = idx
            bright = d["bright"][list(chans)].contiguous()
        return V.ChannelBatch(c, d["u"][sel], d["v"][sel], d["w"][sel], r, lg, mg, ng, bright, snap=d["snap"][sel],
                              pair=d["pair"][sel], sat_pos=d["sat_pos"])

    sub = make(list(range(0, nch, 8)))
    best = V.autotune(sub, use_cache=False)
    report = [{"tuning": vars(tn), "ms": round(ms, 2)} for tn, ms in V.autotune_report(sub)]
    del sub
    b = make(list(range(nch)))
    b.set_tuning(best)
    g = b.graph()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    for _ in range(warmup):
        flush.zero_()  # as in a timed step (see run_ours)
        g.replay()
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier(ws)
        torch.cuda.synchronize()
        t0e.record(st)
        for _ in range(steps):
            flush.zero_()
            g.replay()
        t1e.record(st)
        torch.cuda.synchronize()
        barrier(ws)
    total_ms = max_over_ranks(t0e.elapsed_time(t1e), ws)
    terms_step = 2.0 * K * J
    value = terms_step * steps * ws / (total_ms * 1e-3) / 1e9
    # split of one eager step
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    n0 = L.lib.viss_launch_count()
    e0.record(st)
    b.vis()
    e1.record(st)
    b.recon()
    e2.record(st)
    torch.cuda.synchronize()
    vis_ms, rec_ms = e0.elapsed_time(e1), e1.elapsed_time(e2)
    launches = int(L.lib.viss_launch_count() - n0)
    acc = batch_accuracy(d, b, cfg)
    del b, g
    torch.cuda.empty_cache()
    # the reference's form: one plain launch pair per channel, on 4 channels
    pch = [0, nch // 3, 2 * nch // 3, nch - 1]
    pb = make(pch, cfg.with_(precision=V.PREC_PLAIN))
    pb.step()
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(st)
    pb.step()
    p1.record(st)
    torch.cuda.synchronize()
    pterms = 2.0 * pb.K * J
    plain_value = pterms / (p0.elapsed_time(p1) * 1e-3) / 1e9
    names = {V.PREC_FAST: "fast", V.PREC_COMPENSATED: "compensated"}
    line = {"metric": "Gterms/s batched shaded vis-DFT + recon, 1 GB300", "value": round(value, 3), "unit": UNIT,
            "n_gpus": ws, "steps": steps, "warmup": warmup, "ms_per_step": round(total_ms / steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (fixed-point i32 phase)",
            "data": "synthetic (seeded orbits per channel + Fibonacci sky)",
            "config": {"workload": bw.name, "channels": nch, "K": K, "J": J, "terms_per_step": int(terms_step),
                       "snapshots_per_channel": [int(x) for x in bw.snapshots()], "mask": "geometric",
                       "precision": names.get(prec, str(prec)), "launch": "CUDA graph: 1 persistent vis + 1 "
                       "persistent recon kernel (+ prep)", "l2": "flushed (256 MB write) before each timed step"},
            "vis_ms": round(vis_ms, 2), "recon_ms": round(rec_ms, 2),
            "autotune": {"best": vars(best), "candidates": report, "timed_on": "channels 0, 8, ..., 56"},
            "plain_per_channel": {"value": round(plain_value, 3), "unit": UNIT, "channels": pch,
                                  "what": "PREC_PLAIN, one vis + one recon launch per channel"},
            "speedup_vs_plain": round(value / plain_value, 2), "accuracy": acc, "clocks": clk.summary(),
            "gpu_launches_per_step": launches}
    if sfu_peak:
        dom_ms, dom = (vis_ms, "vis_fast_kernel") if vis_ms >= rec_ms else (rec_ms, "recon_fast_kernel")
        achieved = 2.0 * K * J / (dom_ms * 1e-3) / 1e9
        line["roofline"] = {"bound": "sfu", "kernel": dom, "achieved": round(achieved, 2), "peak": round(sfu_peak, 2),
                            "unit": "G SFU op/s", "frac": round(achieved / sfu_peak, 4),
                            "peak_source": "measured: viss_sfu_probe in this run",
                            "achieved_from": "2 SFU ops x K x J / the pass's CUDA-event time (one eager step)"}
    return line


def batch_accuracy(d, b, cfg):
    """FP64 oracle against the batch on a sample of the 30 MHz channel (the largest
    |uvw|): 32 visibilities x all pixels and 64 pixels x all its visibilities."""
    import numpy as np
    from oracle import oracle as O
    O.build()
    h = lambda t: t.detach().cpu().numpy()  # noqa: E731
    c = b.nch - 1
    r0, r1 = int(b.row_off[c]), int(b.row_off[c + 1])
    u, v, w, snap, pair = (h(d[k][r0:r1]) for k in ("u", "v", "w", "snap", "pair"))
    pos = h(d["sat_pos"])
    K = r1 - r0
    oc = O.make_cfg(mask_mode=O.MASK_GEOMETRIC, phase_scale=cfg.phase_scale, n_offset=cfg.n_offset,
                    occluded_value=cfg.occluded_value, norm=float(b.norm[c]))
    rows = np.linspace(0, K - 1, 32).astype(np.int64)
    Vo = O.vis_dft(oc, u[rows], v[rows], w[rows], d["l"], d["m"], d["n"], h(d["bright"][c]),
                   geo=O.make_geo(pos, snap[rows], pair[rows]), nthreads=O.max_threads())
    Vg = h(b.V[r0:r1])
    pix = np.linspace(0, d["l"].size - 1, 64).astype(np.int64)
    Fo = O.recon(oc, u, v, w, None, Vg, d["l"][pix], d["m"][pix], d["n"][pix], geo=O.make_geo(pos, snap, pair),
                 nthreads=O.max_threads())
    Fg = h(b.F[c])[pix]
    return {"channel": c, "freq_hz": float(d["freqs"][c]),
            "vis_rms": float(np.linalg.norm(Vg[rows] - Vo) / np.linalg.norm(Vo)),
            "recon_rms": float(np.linalg.norm(Fg - Fo) / np.linalg.norm(Fo))}


# ------------------------------------------------------------------ stage 1: orbits -> uvw
def stage1_passes(steps, warmup):
    """Timed passes of stage 1 at the reference's MIncline size (positions, then the
    fused baselines + unique, CUDA events per stage).  Returns (uvw rows, unique rows,
    mean ms per stage, the last pass's tensors)."""
    import torch
    import viss_recon_shade_gb300 as V
    cfg = V.OrbitConfig()
    st = torch.cuda.current_stream()

    def step():
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record(st)
        pos = V.orbit_positions(cfg)
        ev[1].record(st)
        uu, vv, ww = V.unique_uvw(pos, 30.0, ordered=True, capacity=1 << 25)
        ev[2].record(st)
        torch.cuda.synchronize()
        K = pos.shape[0] * pos.shape[1] * (pos.shape[1] - 1)
        return K, uu.numel(), [ev[i].elapsed_time(ev[i + 1]) for i in range(2)], (pos, uu, vv, ww)

    for _ in range(warmup):
        step()
    res = [step() for _ in range(steps)]
    ms = [sum(r[2][i] for r in res) / len(res) for i in range(2)]
    return res[0][0], res[0][1], ms, res[-1][3]


def run_stage1(args, ws, rank, local):
    """--workload stage1: the reference's uvw generation at its own size
    (MIncline_generate_uvw_float.cu: 8 satellites, OrbitRes 864,000, 140 orbits,
    10 MHz): windowed satellite positions, ceil((x_n - x_m) 1e3 / lambda) for the 56
    ordered pairs of 40.32M snapshots = 2.26e9 uvw, then the sort + unique.
    Timed: positions + the fused baselines/unique pass (viss_unique_uvw).  The
    two-call path (viss_baseline_uvw + viss_dedup_uvw, 2.26e9 rows written and
    read back; the pair-major transpose between them untimed) is timed once
    afterwards, checked against the fused result and reported beside it.
    Reported: uvw rows per second, inputs generated on the device.  The shade windows
    of the unique rows (the pipeline's next stage) are timed and reported beside it."""
    import numpy as np
    import torch
    import viss_recon_shade_gb300 as V
    cfg = V.OrbitConfig()  # the reference's constants
    st = torch.cuda.current_stream()
    lam = 30.0
    K, n, ms, (pos, uu, vv, ww) = stage1_passes(args.steps, args.warmup)
    total = sum(ms)
    # the two-call path once, on the last step's positions, checked against the fused result
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record(st)
    u, v, w, snap, pair = V.baseline_uvw(pos, lam, ordered=True, rounding=True)
    del snap, pair
    ev[1].record(st)
    # the reference's pair-major concatenation, as viss_unique_uvw ranks first occurrences
    u, v, w = (x.view(pos.shape[0], -1).t().contiguous().view(-1) for x in (u, v, w))
    ev[1].synchronize()
    base_ms = ev[0].elapsed_time(ev[1])
    V.dedup_uvw(u, v, w)  # once untimed: its workspace (40 bytes a row) comes from the allocator's cache below
    torch.cuda.synchronize()
    ev[1].record(st)
    u2, v2, w2 = V.dedup_uvw(u, v, w)
    ev[2].record(st)
    torch.cuda.synchronize()
    same = all(torch.equal(a.view(torch.int32), b.view(torch.int32)) for a, b in ((uu, u2), (vv, v2), (ww, w2)))
    two = [base_ms, ev[1].elapsed_time(ev[2])]
    del u, v, w, u2, v2, w2
    torch.cuda.empty_cache()
    # stage 2 of the reference's pipeline on this output: the shade windows of every
    # unique uvw at the 10 MHz grid (shade10M: RES 20940), and the oracle's FP32
    # restatement of the reference's kernels on one host thread on a 1M-row sample
    RES = 20940
    V.shade_windows(uu, vv, ww, RES)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(3):
        shade, mean_r = V.shade_windows(uu, vv, ww, RES)
    e1.record(st)
    torch.cuda.synchronize()
    shade_ms = e0.elapsed_time(e1) / 3
    from oracle import oracle as O
    ns = min(n, 1 << 20)
    hu, hv, hw = (x[:ns].cpu().numpy() for x in (uu, vv, ww))
    t0 = time.perf_counter()
    ref, _ = O.shade_windows(hu, hv, hw, RES, mean_r=mean_r, mode=1)
    cpu_s = time.perf_counter() - t0
    diff = np.abs(shade[:ns].cpu().numpy().astype(np.int64) - ref)
    off_by = int((np.minimum(diff, RES - diff) > 0).sum())
    line = {"metric": "uvw rows/s, orbit positions + baseline uvw + sort/unique, 1 GB300",
            "value": round(K / (total * 1e-3) / 1e9, 3), "unit": "G uvw rows/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 positions, int64 keys", "data": "generated on the device",
            "config": {"workload": "stage1", "nsat": cfg.nsat, "orbit_res": cfg.orbit_res,
                       "orbit_counts": cfg.orbit_counts, "snapshots": cfg.snapshots, "uvw_rows": K,
                       "unique_rows": n, "freq_hz": 1e7},
            "stage_ms": {"positions": round(ms[0], 2), "unique_fused": round(ms[1], 2)},
            "two_call_ms": {"baselines": round(two[0], 2), "dedup": round(two[1], 2), "identical": same},
            "shade_windows": {"rows": n, "res": RES, "ms": round(shade_ms, 3),
                              "G_rows_per_s": round(n / (shade_ms * 1e-3) / 1e9, 2),
                              "cpu_baseline": {"value": round(ns / cpu_s / 1e9, 4), "unit": "G rows/s", "cores": 1,
                                               "kind": "port", "sample": f"{ns} rows, FP32 restatement (oracle)"},
                              "window_ends_differing_from_oracle": off_by}}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_textio(args):
    """--workload textio: the reference-format text files of the 10 MHz headline at its
    size, through the library's chunk-parallel reader and writer (viss_text_*, all host
    threads) and the reference's own single-threaded stream loops (restated in the
    oracle: `uvwFile >> u >> v >> w >> freq`, `file << value << std::endl`).
    Read: K = 1,835,008 lines `u v w freq` (integer-valued uvw, as the reference's
    updated_uvw files).  Write: K values one per line (the reference's image-writer
    format, at K lines for a stable timing).  Files live in /dev/shm when it exists, so
    the parse and format are timed, not the disk.  No GPU is used."""
    import ctypes as C
    import shutil
    import tempfile
    import numpy as np
    from viss_recon_shade_gb300 import _lib as L
    from oracle import oracle as O
    K = 1835008
    rng = np.random.default_rng(0)
    cols = np.empty((4, K), np.float32)
    cols[:3] = np.ceil(rng.normal(0, 3000, (3, K)))
    cols[3] = rng.integers(1, 6, K)
    img = (rng.standard_normal(K) * 1e3).astype(np.float32)
    tmp = tempfile.mkdtemp(dir="/dev/shm" if os.path.isdir("/dev/shm") else None)
    try:
        fin, fo1, fo2 = (os.path.join(tmp, n).encode() for n in ("uvw.txt", "F_ours.txt", "F_ref.txt"))
        L.check(L.lib.viss_text_write_floats(fin, 4, cols.ctypes.data_as(C.c_void_p), K, K), "write input")
        in_bytes = os.path.getsize(fin)
        out = np.empty((4, K), np.float32)
        nrows, hv = C.c_int64(0), C.c_int64(0)

        def ours_read():
            L.check(L.lib.viss_text_read_floats(fin, 0, 4, out.ctypes.data_as(C.c_void_p), K, C.byref(nrows),
                                                C.byref(hv)), "viss_text_read_floats")

        def ours_write():
            L.check(L.lib.viss_text_write_floats(fo1, 1, img.ctypes.data_as(C.c_void_p), K, K),
                    "viss_text_write_floats")

        def timed(fn, reps):
            fn()
            t0 = time.perf_counter()
            for _ in range(reps):
                fn()
            return (time.perf_counter() - t0) / reps

        t_read = timed(ours_read, args.steps)
        t_write = timed(ours_write, args.steps)
        ref_cols, nref = O.text_read_stream(fin.decode(), 4, K)
        same_read = nref == K and np.array_equal(ref_cols, out) and np.array_equal(out, cols)
        t_rread = timed(lambda: O.text_read_stream(fin.decode(), 4, K), 1)
        t_rwrite = timed(lambda: O.text_write_stream(fo2.decode(), img), 1)
        with open(fo1, "rb") as a, open(fo2, "rb") as b:
            same_write = a.read() == b.read()
        out_bytes = os.path.getsize(fo1)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    mb = 1e6
    line = {"metric": "reference-format text I/O (parse + format), MB/s of file text", "value":
            round((in_bytes + out_bytes) / (t_read + t_write) / mb, 1), "unit": "MB/s", "n_gpus": 0,
            "steps": args.steps, "warmup": 1, "ms_per_step": round((t_read + t_write) * 1e3, 2),
            "higher_is_better": True, "scaling": "none", "vs_baseline": None, "dtype": "text", "data": "synthetic",
            "config": {"workload": "textio", "read_lines": K, "read_bytes": in_bytes, "write_lines": K,
                       "write_bytes": out_bytes, "threads": os.cpu_count(), "tmpfs": tmp.startswith("/dev/shm")},
            "read": {"ms": round(t_read * 1e3, 2), "MB_per_s": round(in_bytes / t_read / mb, 1),
                     "reference_ms": round(t_rread * 1e3, 2), "identical_values": bool(same_read)},
            "write": {"ms": round(t_write * 1e3, 2), "MB_per_s": round(out_bytes / t_write / mb, 1),
                      "reference_ms": round(t_rwrite * 1e3, 2), "identical_bytes": bool(same_write)},
            "cpu_baseline": {"value": round((in_bytes + out_bytes) / (t_rread + t_rwrite) / mb, 1), "unit": "MB/s",
                             "cores": 1, "kind": "port",
                             "sample": "the same files through the reference's stream loops (oracle)"}}
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.workload == "textio":
        run_textio(args)
        return
    if args.impl == "reference":
        # rank 0 alone runs the reference's CPU implementation (no collective); a GPU
        # only for its ref_cuda_* legs
        rank = int(os.environ.get("RANK", "0"))
        ws, rank, local = dist_setup(group=False, cuda=rank == 0 and not args.no_ref_cuda)
        run_reference(args, ws, rank, local)
        return
    ws, rank, local = dist_setup()
    from viss_recon_shade_gb300.synth import BATCH_WORKLOADS
    if args.workload in BATCH_WORKLOADS:
        run_batch(args, ws, rank, local)
    elif args.workload == "stage1":
        run_stage1(args, ws, rank, local)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
