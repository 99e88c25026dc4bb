"""Benchmark: SimRadar per-pulse emulation loop on one GB300.

One step = one pulse of the emulation loop as simradar runs it
(simradar.c:1011-1074): RS_make_pulse (scatterer signal + range-gate sums)
then RS_advance_time (advection of every scatterer), on the README-scale
workload: 1,998,848 rain scatterers plus 1024 each of leaf, 2x4 board and
brick debris, 40 range gates at 15 m, concept DBU, PPI 3.0 deg, -12..12 deg
at 0.24 deg, PRT 1 ms.  All tables are synthetic and seeded (see
simradar_gb300/synth.py).

  value  pulses/s with the state resident in HBM, timed with CUDA events on
         the worker's stream around each step; L2 is flushed (256 MB write)
         between timed steps, outside the events.
  e2e    the same steps through the C ABI with host buffers: per step the
         beam descriptor goes host->device (kernel parameters) and the pulse
         comes back to pinned host memory, timed on the host clock.
  --impl reference  times the CPU restatement of the reference algorithm
         (the oracle: O(N G) pass 1 + 2-pass reduction, OpenMP on every host
         core) on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

N_RAIN = 1998848
DEBRIS = ((1, 1024), (3, 1024), (6, 1024))
GATES = 40
METRIC = "pulses/s and scatterer-updates/s at 2M scatterers; HBM roofline frac; I/Q err vs FP64"
UNIT = "pulses/s"


def workload_config(n_rain):
    return {
        "workload": "README-scale emulation: %d rain + 3x1024 debris (leaf, 2x4 board, brick), %d gates @ 15 m, "
                    "concept DBU, PPI 3.0 deg -12..12 deg / 0.24 deg, PRT 1 ms, synthetic seeded LES 176x176x80 "
                    "stretched + ADM/RCS 181x91" % (n_rain, GATES),
        "scatterers": n_rain + 3 * 1024,
        "gates": GATES,
        "step": "RS_make_pulse + RS_advance_time (one pulse)",
        "l2": "value: 256 MB L2 flush between timed steps (outside the events); e2e: steps back to back",
    }


def load_peaks():
    p = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def load_traffic(name):
    """Per-launch DRAM bytes of a kernel from a committed ncu summary
    (profiles/<name>.txt, a line 'dram_bytes_per_launch = <int>')."""
    p = os.path.join(HERE, "profiles", name + ".txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            if line.strip().startswith("dram_bytes_per_launch"):
                try:
                    return int(float(line.split("=")[1].split()[0]))
                except Exception:
                    return None
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def cpu_reference(S, pulses, warm=1):
    """The oracle (reference algorithm, every host core) on the workload."""
    from oracle import oracle as O
    st = O.OracleState(S.state)
    t = None
    for k in range(warm + pulses):
        if k == warm:
            t = time.perf_counter()
        sd = S.sd_seq[k % len(S.sd_seq)]
        O.make_pulse(st, S, sd)
        O.advance_time(st, S, S.counts, S.les[0], sd)
    dt = time.perf_counter() - t
    return pulses / dt, O.num_threads()


def build_scene(n_rain):
    from simradar_gb300 import synth
    S = synth.make_scene(num_rain=n_rain, debris=DEBRIS, gates=GATES, les_count=2)
    S.sd_seq = [synth.pulse_sim_desc(S, k, tic=k * 1e-3) for k in range(len(S.scan))]
    return S


def run_reference(args, rank, world):
    if rank != 0:
        return
    S = build_scene(N_RAIN)
    # bounded sample: each step is one full-size pulse; steps capped so the
    # run stays within a few minutes on the host cores
    steps = max(1, min(args.steps, 5))
    warm = max(0, min(args.warmup, 1))
    value, cores = cpu_reference(S, steps, warm)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": steps, "warmup": warm,
        "ms_per_step": 1000.0 / value, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded LES/ADM/RCS tables, see simradar_gb300/synth.py)",
        "config": workload_config(N_RAIN), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "%d full-size pulses (make_pulse + advance_time) after %d warm" % (steps, warm)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "scatterer_updates_per_s": value * S.num_scats,
    }
    print(json.dumps(line))


def run_ours(args, rank, world):
    import ctypes

    from simradar_gb300 import build as B
    from simradar_gb300 import rsc, synth
    B.build()
    import torch
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    S = build_scene(N_RAIN)
    pop = synth.population(S)
    W = rsc.Worker(dev)
    synth.load_worker(W, S)
    stream = torch.cuda.ExternalStream(W.stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    sd_seq = S.sd_seq
    G = S.range_count
    host_pulse = torch.empty((G, 4), dtype=torch.float32).pin_memory()
    hp = host_pulse.numpy()
    gain = float(S.gain)

    def step(k):
        sd = sd_seq[k % len(sd_seq)]
        W.make_pulse(sd)
        W.advance_time(pop, 0, sd)

    # warm-up
    for k in range(args.warmup):
        step(k)
    W.synchronize()

    # device-timed value: per-step events, L2 flushed between steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = W.launch_count
    clocks = ClockSampler(dev)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
            ev[k][0].record(stream)
        W.make_pulse(sd_seq[k % len(sd_seq)])
        ev[k][1].record(stream)
        W.advance_time(pop, 0, sd_seq[k % len(sd_seq)])
        ev[k][2].record(stream)
    W.synchronize()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches = W.launch_count - launches0
    t_pulse = [ev[k][0].elapsed_time(ev[k][1]) for k in range(args.steps)]
    t_adv = [ev[k][1].elapsed_time(ev[k][2]) for k in range(args.steps)]
    total_ms = sum(t_pulse) + sum(t_adv)

    # e2e through the C ABI with host buffers
    W.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        sd = sd_seq[k % len(sd_seq)]
        W.make_pulse(sd)
        W.download_pulse(gain, out=hp)
        W.advance_time(pop, 0, sd)
    W.synchronize()
    e2e_ms = (time.perf_counter() - t0) * 1000.0
    clk = clocks.stop()

    if world > 1:
        t = torch.tensor([total_ms, e2e_ms], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms, e2e_ms = float(t[0]), float(t[1])
    if rank != 0:
        W.close()
        return

    value = world * args.steps / (total_ms / 1000.0)
    e2e = world * args.steps / (e2e_ms / 1000.0)
    peak, peak_kind = load_peaks()
    n_deb = sum(c for _, c in DEBRIS)
    adv_bytes = 64 * N_RAIN + 128 * n_deb
    pulse_bytes = 32 * (N_RAIN + n_deb) + 16 * G
    adv_ms = statistics.mean(t_adv)
    pul_ms = statistics.mean(t_pulse)
    adv_gbs = adv_bytes / (adv_ms * 1e-3) / 1e9
    pul_gbs = pulse_bytes / (pul_ms * 1e-3) / 1e9
    if adv_ms >= pul_ms:
        dom = {"kernel": "k_advance", "achieved": adv_gbs, "traffic": load_traffic("k_advance_traffic")}
        other = {"kernel": "k_pulse<0>", "achieved": pul_gbs, "ms": pul_ms, "bytes_per_launch": pulse_bytes}
        dom_bytes = adv_bytes
    else:
        dom = {"kernel": "k_pulse<0>", "achieved": pul_gbs, "traffic": load_traffic("k_pulse_traffic")}
        other = {"kernel": "k_advance", "achieved": adv_gbs, "ms": adv_ms, "bytes_per_launch": adv_bytes}
        dom_bytes = pulse_bytes
    roofline = {"bound": "hbm", "achieved": dom["achieved"], "peak": peak, "unit": "GB/s",
                "frac": dom["achieved"] / peak, "traffic": dom["traffic"], "kernel": dom["kernel"],
                "algorithmic_bytes_per_launch": dom_bytes, "peak_kind": peak_kind, "other_kernel": other}
    # CPU baseline: the oracle on a bounded sample of the same workload
    cpu = None
    if not args.no_cpu_baseline:
        W.close()
        cpu_value, cores = cpu_reference(S, pulses=12, warm=1)
        cpu = {"value": cpu_value, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "12 full-size pulses (make_pulse + advance_time) after 1 warm, OpenMP on all host cores"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded LES/ADM/RCS tables, see simradar_gb300/synth.py)",
        "config": workload_config(N_RAIN),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 64, "d2h_bytes_per_step": G * 16},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": int(launches),
        "scatterer_updates_per_s": value * S.num_scats,
        "kernel_ms": {"k_pulse<0>": pul_ms, "k_advance": adv_ms},
    }
    print(json.dumps(line))
    if args.no_cpu_baseline:
        W.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
