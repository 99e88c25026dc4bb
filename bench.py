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
         comes back to pinned host memory (queued in stream order, the gain
         applied on the host at the end), timed on the host clock;
         blocking_read_value waits for every pulse before the next step.
  --impl reference  times the CPU restatement of the reference algorithm
         (the oracle: O(N G) pass 1 + 2-pass reduction, OpenMP on every host
         core) on the same workload.

Extra sections on one GPU (added to the same JSON line):
  precision  8,388,608 scatterers with the box and gates 30 km out: plain and
             compensated pulses against the FP64 pulse of the same state
             (per-gate relative I/Q error, Zdr / rhohv bias over the pulse
             series) and the throughput of each form.
  batch      64 instances (scatterers log-uniform 65,536-4,194,304, debris
             0-4096 per type, N0 4000-16000, PPI / RHI mix) in the
             compensated form: batched (three launches per step for all, CUDA
             graph, autotuned pulse shape) against the same instances run back
             to back one after another.
  les        the LES frame swap inside the loop: no swap, the reference's
             (host remap + blocking upload of uvwt / cpxx), and the frame
             source (raw planes on the copy stream, remapped on the device).
  large      33,554,432 rain + 131,072 debris, LES 352x352x160, RHI
             0.5-20 deg at 0.02 deg, compensated form, I/Q streamed to pinned
             host buffers every 100 pulses and on to a .iq file by the
             backend's background writer, one LES slot refilled on the copy
             stream during the run.
  small      the reference's CPU-runnable case: 131,072 rain (DBU), the
             same PPI, 100 pulses -- on the GPU through the C ABI (every
             pulse copied back) and on the host cores with the oracle after
             one warm pulse.
"""
import argparse
import json
import math
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
SECTIONS = ("precision", "batch", "les", "large", "small")
SORT_INTERVAL = 128   # the backend's default (rsc_set_sort_interval)


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


def cpu_model():
    """The host CPU's model name (lscpu), for the CPU baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip() + " (%s, %d logical CPUs)" % (os.uname().machine, os.cpu_count())
    except Exception:
        pass
    return "%s, %d logical CPUs" % (os.uname().machine, os.cpu_count())


def build_scene(n_rain):
    from simradar_gb300 import synth
    S = synth.make_scene(num_rain=n_rain, debris=DEBRIS, gates=GATES, les_count=2)
    S.sd_seq = [synth.pulse_sim_desc(S, k, tic=k * 1e-3) for k in range(len(S.scan))]
    return S


def traffic_bytes(n_rain, n_deb, gates):
    """Algorithmic HBM bytes per launch.  Advance: the persistent state, read
    and written once -- rain pos and vel (64 B), debris pos, ori, vel and tum
    (128 B); the RCS, which the kernels also store (16 B more per scatterer)
    but which is a function of the state, the respawn seeds and the LES /
    table texels (reused across scatterers, L2 resident) are not counted.
    Pulse: position and complex H/V signal source read once (32 B) and the
    gates written."""
    adv = 64 * n_rain + 128 * n_deb
    pul = 32 * (n_rain + n_deb) + 16 * gates
    return adv, pul


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
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "cpu": cpu_model(),
                         "sample": "%d full-size pulses (make_pulse + advance_time) after %d warm" % (steps, warm)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "scatterer_updates_per_s": value * S.num_scats,
    }
    print(json.dumps(line))


def max_over_ranks(torch, values, world, device):
    """The slowest rank's timings (element-wise max over ranks)."""
    if world <= 1:
        return [float(v) for v in values]
    t = torch.tensor(values, dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(v) for v in t]


def whole_job_rate(world, steps, ms):
    """Pulses per second of the whole job: every replica forms `steps`
    pulses; the time is the slowest replica's."""
    return world * steps / (ms / 1000.0)


def timed_steps(torch, W, pop, sd_seq, steps, flush=None, les_id=0):
    """Per-step (step ms, pulse ms, advance ms) with CUDA events.  The pulse
    runs on the worker's stream and the advance of the same step beside it
    on the advance stream: a step is timed from an event on the worker's
    stream, which the advance stream also waits for, to an event recorded
    after the worker's stream has waited for the advance stream; the pulse
    and the advance are timed on their own streams.  `flush` (a device
    tensor larger than L2) is rewritten between steps, outside the events."""
    main = torch.cuda.ExternalStream(W.stream)
    adv = torch.cuda.ExternalStream(W.advance_stream)
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(steps)]
    torch.cuda.synchronize()
    for k in range(steps):
        if flush is not None:
            with torch.cuda.stream(main):
                flush.fill_(float(k))
        e = ev[k]
        e[0].record(main)
        adv.wait_event(e[0])
        W.make_pulse(sd_seq[k % len(sd_seq)])
        e[1].record(main)
        e[2].record(adv)
        W.advance_time(pop, les_id, sd_seq[k % len(sd_seq)])
        e[3].record(adv)
        main.wait_stream(adv)
        e[4].record(main)
    W.synchronize()
    torch.cuda.synchronize()
    t_step = [ev[k][0].elapsed_time(ev[k][4]) for k in range(steps)]
    t_pulse = [ev[k][0].elapsed_time(ev[k][1]) for k in range(steps)]
    t_adv = [ev[k][2].elapsed_time(ev[k][3]) for k in range(steps)]
    return t_step, t_pulse, t_adv


# ------------------------------------------------------------------ precision
def gate_stats(series):
    """Zdr (dB) and rhohv per gate from a (pulses, gates, 4) I/Q series."""
    s = series.astype(np.float64)
    h = s[..., 0] + 1j * s[..., 1]
    v = s[..., 2] + 1j * s[..., 3]
    ph = (np.abs(h) ** 2).sum(axis=0)
    pv = (np.abs(v) ** 2).sum(axis=0)
    ok = (ph > 0) & (pv > 0)
    zdr = np.where(ok, 10.0 * np.log10(np.where(ok, ph, 1.0) / np.where(ok, pv, 1.0)), 0.0)
    rho = np.where(ok, np.abs((h * np.conj(v)).sum(axis=0)) / np.sqrt(np.where(ok, ph * pv, 1.0)), 0.0)
    return zdr, rho, ok


EPS_REL = 1.0e-2


def iq_errors(got, ref):
    """Per-gate complex relative error |got - ref| / max(|ref|, eps) for H and
    V, eps = EPS_REL x the RMS gate magnitude of the same pulse and
    polarisation.  Gate values are sums of many terms of random phase, so
    |ref| is Rayleigh distributed and a few gates of a long series fall near
    zero, where any absolute error is a large relative one; eps (40 dB below
    the typical gate) keeps those from setting the maximum.  max_rel_raw is
    the same without eps."""
    g = got.astype(np.float64)
    r = ref.astype(np.float64)
    e_h = np.hypot(g[..., 0] - r[..., 0], g[..., 1] - r[..., 1])
    e_v = np.hypot(g[..., 2] - r[..., 2], g[..., 3] - r[..., 3])
    m_h = np.hypot(r[..., 0], r[..., 1])
    m_v = np.hypot(r[..., 2], r[..., 3])
    eps_h = EPS_REL * np.sqrt((m_h ** 2).mean(axis=-1, keepdims=True))
    eps_v = EPS_REL * np.sqrt((m_v ** 2).mean(axis=-1, keepdims=True))
    e = np.concatenate([e_h.ravel(), e_v.ravel()])
    m = np.concatenate([m_h.ravel(), m_v.ravel()])
    den = np.concatenate([np.maximum(m_h, eps_h).ravel(), np.maximum(m_v, eps_v).ravel()])
    nz = den > 0
    rel = e[nz] / den[nz]
    raw = e[m > 0] / m[m > 0]
    return {"max_rel": float(rel.max()), "rms_rel": float(np.sqrt((rel ** 2).mean())),
            "p99_rel": float(np.percentile(rel, 99)), "max_rel_raw": float(raw.max()),
            "within_1e-5": float((rel <= 1.0e-5).mean()), "eps": "%g x RMS gate magnitude" % EPS_REL,
            "values": int(rel.size), "above_1e-5": int((rel > 1.0e-5).sum()),
            "p999_rel": float(np.percentile(rel, 99.9)),
            "abs_err_over_rms_max": float(e.max() / max(float(np.sqrt((m ** 2).mean())), 1e-300))}


def bench_precision(torch, rsc, synth, dev, steps, n_err=2000):
    n = 8388608
    S = synth.make_scene(num_rain=n, gates=GATES, les_count=1, range_offset=30000.0, seed=4242,
                         scan=synth.ppi_positions(0.7, -0.6, 0.6, 0.012))
    sd_seq = [synth.pulse_sim_desc(S, k, tic=k * 1e-3) for k in range(len(S.scan))]
    pop = synth.population(S)
    W = rsc.Worker(dev)
    synth.load_worker(W, S)
    S.state = None
    got = {m: np.zeros((n_err, GATES, 4), np.float32) for m in (0, 1, 2)}
    t_err = time.perf_counter()
    for k in range(n_err):
        sd = sd_seq[k % len(sd_seq)]
        for m in (2, 1, 0):
            W.set_precision(m)
            W.make_pulse(sd)
            W.download_pulse(1.0, out=got[m][k])
        W.advance_time(pop, 0, sd)
    t_err = time.perf_counter() - t_err
    z64, r64, ok = gate_stats(got[2])
    out = {"workload": "8,388,608 rain, box and 40 gates 30 km out (gates from 31,850 m), PPI 0.7 deg "
                       "-0.6..0.6 deg / 0.012 deg, concept DBU; errors over %d pulses against the FP64 pulse "
                       "(RSC_PULSE_F64) of the same state" % n_err}
    for m, name in ((1, "compensated"), (0, "plain")):
        z, r, _ = gate_stats(got[m])
        e = iq_errors(got[m], got[2])
        e["zdr_bias_db_max"] = float(np.abs(z - z64)[ok].max()) if ok.any() else None
        e["rhohv_bias_max"] = float(np.abs(r - r64)[ok].max()) if ok.any() else None
        out[name] = e
    timing = {}
    for m, name in ((0, "plain"), (1, "compensated")):
        W.set_precision(m)
        for k in range(3):
            W.make_pulse(sd_seq[k])
            W.advance_time(pop, 0, sd_seq[k])
        ts, tp, ta = timed_steps(torch, W, pop, sd_seq, steps)
        timing[name] = {"pulses_per_s": steps / (sum(ts) / 1000.0), "step_ms": statistics.mean(ts),
                        "pulse_ms": statistics.mean(tp), "advance_ms": statistics.mean(ta)}
    out["throughput"] = timing
    out["timed_steps"] = steps
    out["error_pulses"] = n_err
    out["error_run_s"] = t_err
    W.close()
    return out


# ---------------------------------------------------------------------- batch
def bench_batch(torch, rsc, synth, dev, steps):
    count = 64
    scenes = synth.batch_workload(count, gates=GATES)
    ws = []
    for S in scenes:
        W = rsc.Worker(dev)
        synth.load_worker(W, S)
        W.set_precision(rsc.PULSE_COMPENSATED)
        S.state = None
        ws.append(W)
    pops = [synth.population(S) for S in scenes]
    total = sum(S.num_scats for S in scenes)

    def sims(k0, K):
        a = np.zeros((K, count, 16), np.float32)
        for j in range(K):
            for i, S in enumerate(scenes):
                a[j, i] = synth.pulse_sim_desc(S, k0 + j, tic=(k0 + j) * 1e-3)
        return a

    B = rsc.Batch(ws)
    B.set_populations(pops)
    B.set_precision(rsc.PULSE_COMPENSATED)
    shape = B.autotune(sims(0, 1)[0])
    adv_shape = B.advance_shape
    les = np.zeros((steps, count), np.int32)
    out = np.empty((steps, count, B.max_gates, 4), np.float32)
    bstream = torch.cuda.ExternalStream(B.stream)
    res = {}
    for form in ("graph", "stream", "persistent"):
        use_graph = form == "graph"
        B.set_persistent(form == "persistent")
        B.run(sims(0, steps), les, out=out, use_graph=use_graph)       # warm-up (and graph capture)
        sd = sims(steps, steps)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        B.synchronize()
        l0 = B.launch_count
        t0 = time.perf_counter()
        e0.record(bstream)
        B.run(sd, les, out=out, use_graph=use_graph)
        e1.record(bstream)
        wall = time.perf_counter() - t0
        e1.synchronize()
        dev_ms = e0.elapsed_time(e1)
        key = "batched_" + form
        res[key] = {"pulses_per_s": count * steps / wall, "device_pulses_per_s": count * steps / (dev_ms / 1e3),
                    "launches": B.launch_count - l0}
    B.close()
    # back to back: each instance runs its steps alone, one after another
    hp = torch.empty((GATES, 4), dtype=torch.float32).pin_memory().numpy()
    for W, S, p in zip(ws, scenes, pops):
        for k in range(2):
            sd = synth.pulse_sim_desc(S, k)
            W.make_pulse(sd)
            W.advance_time(p, 0, sd)
    torch.cuda.synchronize()
    seqs = [[synth.pulse_sim_desc(S, k, tic=k * 1e-3) for k in range(steps)] for S in scenes]
    ring = torch.empty((steps, GATES, 4), dtype=torch.float32).pin_memory().numpy()

    def back_to_back(copy):
        t0 = time.perf_counter()
        for W, seq, p in zip(ws, seqs, pops):
            for k in range(steps):
                W.make_pulse(seq[k])
                if copy == "async":
                    W.download_pulse_async(ring[k])
                elif copy == "blocking":
                    W.download_pulse(1.0, out=hp)
                W.advance_time(p, 0, seq[k])
            W.synchronize()
        return time.perf_counter() - t0

    wall_async = back_to_back("async")
    wall_blocking = back_to_back("blocking")
    wall_none = back_to_back("none")
    for W in ws:
        W.close()
    res["back_to_back"] = {"pulses_per_s": count * steps / wall_async,
                           "pulses_per_s_blocking_read": count * steps / wall_blocking,
                           "pulses_per_s_no_download": count * steps / wall_none}
    best = max(("batched_graph", "batched_persistent"), key=lambda k: res[k]["pulses_per_s"])
    res["batched_form"] = best
    res["persistent_vs_graph"] = res["batched_persistent"]["pulses_per_s"] / res["batched_graph"]["pulses_per_s"]
    bg = res[best]["pulses_per_s"]
    res["speedup_vs_back_to_back"] = bg / res["back_to_back"]["pulses_per_s"]
    res["speedup_vs_back_to_back_blocking_read"] = bg / res["back_to_back"]["pulses_per_s_blocking_read"]
    res["speedup_vs_back_to_back_no_download"] = bg / res["back_to_back"]["pulses_per_s_no_download"]
    res["workload"] = ("64 instances, scatterers log-uniform 65,536-4,194,304 (total %d), debris 0-4096 per type, "
                       "Marshall-Palmer N0 4000-16000, PPI / RHI alternating, %d gates, compensated form; %d steps "
                       "timed per instance.  Every pulse reaches the host in both: batched, one copy per run; back "
                       "to back, each pulse copied to page-locked memory in stream order with one wait per "
                       "instance (speedup_vs_back_to_back).  Secondary: back to back with a blocking read of every "
                       "pulse as rs.c does, and with no pulse copied" % (total, GATES, steps))
    res["pulse_shape"] = {"warps": shape[0], "blocks_per_sm": shape[1]}
    res["advance_shape"] = {"threads": adv_shape[0], "blocks_per_sm": adv_shape[1] or "all that fit"}
    res["scatterer_updates_per_s"] = bg / count * total
    return res


# ---------------------------------------------------------------------- large
def bench_large(torch, rsc, synth, dev, chunks, chunk=100):
    import shutil
    import tempfile

    from simradar_gb300 import iqfile
    n_rain = 33554432
    cfg = synth.LESConfig(nx=352, ny=352, nz=160)
    debris = [(synth.OBJ_LEAF, 43691), (synth.OBJ_WOODBOARD_2X4, 43691), (synth.OBJ_BRICK, 43690)]
    S = synth.make_scene(num_rain=n_rain, debris=debris, gates=GATES, les_cfg=cfg, les_count=2, seed=777,
                         scan=synth.rhi_positions(0.0, 0.5, 20.0, 0.02))
    pop = synth.population(S)
    W = rsc.Worker(dev)
    synth.load_worker(W, S, les_slot_volumes=(0,))
    W.set_precision(rsc.PULSE_COMPENSATED)
    nscat = S.num_scats
    S.state = None
    # the LES frames in page-locked memory for the refills: frame f of the
    # run is the synthetic volume f % 2 (two volumes of the recipe alternate)
    nxt = S.les[1]
    pinned = [(torch.from_numpy(np.ascontiguousarray(v.uvwt)).pin_memory(),
               torch.from_numpy(np.ascontiguousarray(v.cpxx)).pin_memory()) for v in S.les[:2]]
    tp = float(S.les_cfg.tp)
    # chunk c forms pulses chunk (c + 1) ... (the first chunk is the warm-up run)
    frame_of = [int(math.floor((c + 1) * chunk * float(S.prt) / tp + 1e-9)) for c in range(chunks + 1)]
    B = rsc.Batch([W])
    B.set_populations([pop])
    B.set_precision(rsc.PULSE_COMPENSATED)
    ring = [torch.empty((chunk, 1, B.max_gates, 4), dtype=torch.float32).pin_memory() for _ in range(2)]
    stream = torch.cuda.ExternalStream(B.stream)
    tmpdir = tempfile.mkdtemp(prefix="simradar_iq_")
    iq_path = os.path.join(tmpdir, "large.iq")
    params = {"c": 3.0e8, "prt": float(S.prt), "lambda": float(S.lam), "tx_power_watt": 50.0e3,
              "antenna_gain_dbi": 44.5, "antenna_bw_deg": 1.0, "tau": 0.2e-6, "range_start": float(S.range_start),
              "range_end": float(S.range_start + S.range_delta * (GATES - 1)), "range_delta": float(S.range_delta),
              "elevation_start_deg": 0.5, "elevation_end_deg": 20.0, "elevation_delta_deg": 0.02,
              "prf": 1.0 / float(S.prt), "dr": float(S.dr), "range_count": GATES}
    writer = iqfile.IQWriter(iq_path, params, counts=S.counts, scan_mode="RHI", scan_start=0.5, scan_end=20.0,
                             scan_delta=0.02, seed=777)

    def sims(k0):
        a = np.zeros((chunk, 1, 16), np.float32)
        for j in range(chunk):
            a[j, 0] = synth.pulse_sim_desc(S, k0 + j, tic=(k0 + j) * 1e-3)
        return a

    def les_ids(slot):
        return np.full((chunk, 1), slot, np.int32)

    def beam(k0):
        el = np.array([S.scan[(k0 + j) % len(S.scan)][1] for j in range(chunk)], np.float32)
        az = np.array([S.scan[(k0 + j) % len(S.scan)][0] for j in range(chunk)], np.float32)
        return (np.arange(k0, k0 + chunk, dtype=np.float32) * np.float32(S.prt)), el, az

    B.autotune(sims(0)[0])
    B.run(sims(0), les_ids(0), out=ring[0].numpy())     # warm-up and graph capture
    B.synchronize()
    done = [None, None]
    t0 = time.perf_counter()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    swaps = 0

    def drain(r):
        ev, c = done[r]
        ev.synchronize()
        t, el, az = beam(chunk * (c + 1))
        writer.write(ring[r].numpy()[:, 0], times=t, el_deg=el, az_deg=az, gain=float(S.gain))
        done[r] = None

    for c in range(chunks):
        r = c % 2
        if done[r] is not None:
            drain(r)
        # the frame of this chunk's simulation time (a new one every tp, as
        # RS_advance_time swaps, rs.c:5188-5200) in slot frame % 2
        slot = frame_of[c] % 2
        B.run(sims(chunk * (c + 1)), les_ids(slot), out=ring[r].numpy(), wait=False)
        ev = torch.cuda.Event()
        ev.record(stream)
        done[r] = (ev, c)
        if frame_of[c + 1] != frame_of[c] and c + 1 < chunks:
            # the next frame into the other slot while this chunk runs
            f = frame_of[c + 1]
            u, cp = pinned[f % 2]
            B.set_les_async(0, f % 2, u.numpy(), cp.numpy())
            swaps += 1
    e1.record(stream)
    for r in (chunks % 2, (chunks + 1) % 2):
        if done[r] is not None:
            drain(r)
    B.synchronize()
    writer.flush()
    wall = time.perf_counter() - t0
    dev_ms = e0.elapsed_time(e1)
    writer.close()
    pulses = chunks * chunk
    # RS_populate's initial state for the same population, made on the host
    # and copied in overlapped blocks (what a session start costs)
    pa = rsc.PopulateArgs.make(19760520, S.concept, S.box[:3], S.box[3:], S.counts, S.dsd_r, S.dsd_cdf)
    t1 = time.perf_counter()
    rsc.populate_upload(W, pa)
    populate_s = time.perf_counter() - t1
    d = iqfile.read_iq(iq_path)
    shutil.rmtree(tmpdir, ignore_errors=True)
    B.close()
    W.close()
    iq = d["iq"]
    return {"workload": "33,554,432 rain + 131,072 debris (leaf / 2x4 board / brick), LES 352x352x160, RHI 0.5-20 "
                        "deg / 0.02 deg (976 positions, repeated), %d gates, compensated form; %d pulses at PRT 1 ms "
                        "in chunks of %d streamed to pinned host buffers and on to a .iq file (background writer); "
                        "a new LES frame every tp = %g s of simulation time (les.c:170), %d swaps, each frame "
                        "(2 x %d MB, two synthetic volumes alternating) refilled on the copy stream into the "
                        "inactive slot during the chunk before it is used" % (
                            GATES, pulses, chunk, tp, swaps, int(nxt.uvwt.nbytes / 1e6)),
            "les_swaps": swaps,
            "pulses_per_s": pulses / wall, "device_pulses_per_s": pulses / (dev_ms / 1e3),
            "scatterer_updates_per_s": pulses / wall * nscat, "pulses": pulses,
            "populate_s": populate_s,
            "iq_file_pulses": int(iq.shape[0]), "iq_finite": bool(np.isfinite(iq).all()),
            "iq_nonzero_pulses": int((np.abs(iq).sum(axis=(1, 2)) > 0).sum())}


def bench_les(torch, rsc, synth, dev, S, steps=2000, period=100, repeats=3):
    """The LES frame swap inside the pulse loop (rs.c:5188-5200): every
    `period` steps the next frame goes into the inactive slot and the loop
    moves to it.  Three ways on the README workload: no swap; the reference's
    (the frame already remapped on the host, as les.c's background thread
    leaves it, then a blocking upload of uvwt + cpxx from pageable memory,
    RS_set_vel_data); and the frame source (raw planes read ahead, copied on
    the copy stream and remapped on the device, overlapped with the loop)."""
    import shutil
    import tempfile
    tmpdir = tempfile.mkdtemp(prefix="simradar_les_")
    frames = 4
    synth.write_les_folder(tmpdir, S.les_cfg, [S.les[k % len(S.les)] for k in range(frames)])
    src = rsc.LESSource(tmpdir, "suctvort")
    pop = synth.population(S)
    W = rsc.Worker(dev)
    synth.load_worker(W, S)
    stream = torch.cuda.ExternalStream(W.stream)
    sd_seq = S.sd_seq
    for k in range(3):
        W.make_pulse(sd_seq[k])
        W.advance_time(pop, 0, sd_seq[k])
    W.synchronize()

    def loop(mode):
        slot, frame = 0, 0
        upload_s = []
        W.synchronize()
        t0 = time.perf_counter()
        for k in range(steps):
            if mode != "none" and k % period == period - 1:
                frame = (frame + 1) % frames
                t1 = time.perf_counter()
                if mode == "source":
                    src.upload_async(W, 1 - slot, frame)
                else:
                    uvwt, cpxx = host_frames[frame]
                    W.set_les(1 - slot, uvwt, cpxx, S.les_desc)
                upload_s.append(time.perf_counter() - t1)
            if mode != "none" and k % period == 0 and k > 0:
                slot = 1 - slot
            W.make_pulse(sd_seq[k % len(sd_seq)])
            W.advance_time(pop, slot, sd_seq[k % len(sd_seq)])
        W.synchronize()
        return (time.perf_counter() - t0) * 1e3 / steps, (statistics.mean(upload_s) * 1e3 if upload_s else 0.0)

    # the reference's frames arrive remapped by les.c's background thread
    host_frames = [src.read(f)[:2] for f in range(frames)]
    loop("source")   # page the frames in, pin the source's buffers
    # the three loops interleaved, each run `repeats` times: the median of
    # each (the loop is timed on the host clock, which a busy host jolts)
    runs = {"none": [], "blocking": [], "source": []}
    for _ in range(repeats):
        for mode in ("none", "blocking", "source"):
            runs[mode].append(loop(mode))
    none_ms = statistics.median(r[0] for r in runs["none"])
    ref_ms = statistics.median(r[0] for r in runs["blocking"])
    ref_call = statistics.median(r[1] for r in runs["blocking"])
    src_ms = statistics.median(r[0] for r in runs["source"])
    src_call = statistics.median(r[1] for r in runs["source"])
    W.close()
    src.close()
    shutil.rmtree(tmpdir, ignore_errors=True)
    nn = S.les_cfg.nx * S.les_cfg.ny * S.les_cfg.nz
    swaps = steps // period
    return {"workload": "README loop (2M scatterers), LES %dx%dx%d, a frame swap every %d steps, %d steps, "
                        "each way run %d times interleaved (medians)"
                        % (S.les_cfg.nx, S.les_cfg.ny, S.les_cfg.nz, period, steps, repeats),
            "runs_ms_per_step": {k: [r[0] for r in v] for k, v in runs.items()},
            "ms_per_step_no_swap": none_ms,
            "ms_per_step_blocking_swap": ref_ms, "blocking_swap_call_ms": ref_call,
            "ms_per_step_source_swap": src_ms, "source_swap_call_ms": src_call,
            "swap_cost_ms_blocking": (ref_ms - none_ms) * steps / swaps,
            "swap_cost_ms_source": (src_ms - none_ms) * steps / swaps,
            "h2d_bytes_per_swap_blocking": nn * 32, "h2d_bytes_per_swap_source": nn * 20}


def bench_small(torch, rsc, synth, dev, pulses=100):
    """The reference's CPU-runnable configuration: 131,072 rain scatterers
    (concept DBU), PPI 3.0 deg, -12..12 deg at 0.24 deg, 40 gates at 15 m,
    100 pulses.  GPU: the pulses through the C ABI with every pulse copied to
    pinned host memory (host clock, after three warm pulses).  CPU: the
    oracle (every host core) on the same 100 pulses after one warm pulse."""
    S = synth.make_scene(num_rain=131072, gates=GATES, les_count=1)
    S.sd_seq = [synth.pulse_sim_desc(S, k, tic=k * 1e-3) for k in range(len(S.scan))]
    pop = synth.population(S)
    W = rsc.Worker(dev)
    synth.load_worker(W, S)
    ring = torch.empty((pulses, GATES, 4), dtype=torch.float32).pin_memory()
    ring_np = ring.numpy()
    for k in range(3):
        W.make_pulse(S.sd_seq[k])
        W.advance_time(pop, 0, S.sd_seq[k])
    W.synchronize()
    t0 = time.perf_counter()
    for k in range(pulses):
        sd = S.sd_seq[k % len(S.sd_seq)]
        W.make_pulse(sd)
        W.download_pulse_async(ring_np[k])
        W.advance_time(pop, 0, sd)
    W.synchronize()
    gpu_s = time.perf_counter() - t0
    W.close()
    cpu_value, cores = cpu_reference(S, pulses=pulses, warm=1)
    return {"workload": "131,072 rain, concept DBU, PPI 3.0 deg -12..12 deg / 0.24 deg, %d gates @ 15 m, "
                        "%d pulses" % (GATES, pulses),
            "gpu_pulses_per_s": pulses / gpu_s, "cpu_pulses_per_s": cpu_value, "cpu_cores": cores,
            "cpu": cpu_model(), "gpu_over_cpu": (pulses / gpu_s) / cpu_value,
            "note": "GPU through the C ABI with every pulse copied to pinned host memory (host clock); CPU: "
                    "the oracle on the same pulses after one warm pulse"}


def run_ours(args, rank, world):
    from simradar_gb300 import build as Bld
    from simradar_gb300 import rsc, synth
    Bld.build()
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

    # warm-up
    for k in range(args.warmup):
        W.make_pulse(sd_seq[k % len(sd_seq)])
        W.advance_time(pop, 0, sd_seq[k % len(sd_seq)])
    W.synchronize()

    # the periodic spatial sort (every `interval` advances): its cost per sort,
    # from steps that each sort (interval 1) against steps that do not
    interval = SORT_INTERVAL
    W.set_sort_interval(1)
    ts_sort, _, _ = timed_steps(torch, W, pop, sd_seq, 8, flush=flush)
    W.set_sort_interval(0)
    ts_plain, _, _ = timed_steps(torch, W, pop, sd_seq, 8, flush=flush)
    W.set_sort_interval(interval)
    sort_ms = max(0.0, statistics.median(ts_sort) - statistics.median(ts_plain))

    # device-timed value: per-step events, L2 flushed between steps
    launches0 = W.launch_count
    sorts0 = W.sort_count
    clocks = ClockSampler(dev)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    t_step, t_pulse, t_adv = timed_steps(torch, W, pop, sd_seq, args.steps, flush=flush)
    if world > 1:
        torch.distributed.barrier()
    launches = W.launch_count - launches0
    sorts_value = W.sort_count - sorts0
    # value carries the sort's amortised cost whatever the window holds: the
    # sorts that fell in it are taken out and steps / interval of them put in
    total_ms = sum(t_step) + (args.steps / interval - sorts_value) * sort_ms

    # e2e through the C ABI with host buffers: every step's pulse is copied to
    # page-locked host memory in stream order (the host queues the next steps
    # meanwhile) and the gain is applied on the host once the copies are in
    ring = torch.empty((args.steps, G, 4), dtype=torch.float32).pin_memory()
    ring_np = ring.numpy()
    W.synchronize()
    sorts0 = W.sort_count
    t0 = time.perf_counter()
    for k in range(args.steps):
        sd = sd_seq[k % len(sd_seq)]
        W.make_pulse(sd)
        W.download_pulse_async(ring_np[k])
        W.advance_time(pop, 0, sd)
    W.synchronize()
    ring_np *= np.float32(gain)
    e2e_ms = (time.perf_counter() - t0) * 1000.0
    sorts_e2e = W.sort_count - sorts0
    e2e_ms += (args.steps / interval - sorts_e2e) * sort_ms
    # the same with a blocking read of every pulse before the next step, as
    # rs.c reads them (clEnqueueReadBuffer + wait per pulse)
    W.synchronize()
    sorts0 = W.sort_count
    t0 = time.perf_counter()
    for k in range(args.steps):
        sd = sd_seq[k % len(sd_seq)]
        W.make_pulse(sd)
        W.download_pulse(gain, out=hp)
        W.advance_time(pop, 0, sd)
    W.synchronize()
    e2e_blocking_ms = (time.perf_counter() - t0) * 1000.0
    e2e_blocking_ms += (args.steps / interval - (W.sort_count - sorts0)) * sort_ms
    clk = clocks.stop()

    total_ms, e2e_ms, e2e_blocking_ms = max_over_ranks(torch, [total_ms, e2e_ms, e2e_blocking_ms], world, "cuda")
    if rank != 0:
        W.close()
        return

    value = whole_job_rate(world, args.steps, total_ms)
    e2e = whole_job_rate(world, args.steps, e2e_ms)
    e2e_blocking = whole_job_rate(world, args.steps, e2e_blocking_ms)
    peak, peak_kind = load_peaks()
    n_deb = sum(c for _, c in DEBRIS)
    adv_bytes, pulse_bytes = traffic_bytes(N_RAIN, n_deb, G)
    adv_ms = statistics.mean(t_adv)
    pul_ms = statistics.mean(t_pulse)
    adv_gbs = adv_bytes / (adv_ms * 1e-3) / 1e9
    pul_gbs = pulse_bytes / (pul_ms * 1e-3) / 1e9
    if adv_ms >= pul_ms:
        dom = {"kernel": "k_advance_rain + k_advance_debris", "achieved": adv_gbs,
               "traffic": load_traffic("k_advance_readme_2m")}
        other = {"kernel": "k_pulse_group<0, 2, 1>", "achieved": pul_gbs, "ms": pul_ms, "bytes_per_launch": pulse_bytes,
                 "frac": pul_gbs / peak}
        dom_bytes = adv_bytes
    else:
        dom = {"kernel": "k_pulse_group<0, 2, 1>", "achieved": pul_gbs, "traffic": load_traffic("k_pulse_readme_2m")}
        other = {"kernel": "k_advance_rain + k_advance_debris", "achieved": adv_gbs, "ms": adv_ms,
                 "bytes_per_launch": adv_bytes,
                 "frac": adv_gbs / peak}
        dom_bytes = pulse_bytes
    step_ms = total_ms / args.steps
    step_gbs = (adv_bytes + pulse_bytes) / (step_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "achieved": dom["achieved"], "peak": peak, "unit": "GB/s",
                "frac": dom["achieved"] / peak, "traffic": dom["traffic"], "kernel": dom["kernel"],
                "algorithmic_bytes_per_launch": dom_bytes, "peak_kind": peak_kind, "other_kernel": other,
                "step": {"note": "the pulse and the advance share the GPU within a step (two streams): their "
                                 "algorithmic bytes over the step time",
                         "bytes": adv_bytes + pulse_bytes, "ms": step_ms, "achieved": step_gbs,
                         "frac": step_gbs / peak}}

    # the compensated form on the same workload
    W.set_precision(rsc.PULSE_COMPENSATED)
    csteps = min(args.steps, 100)
    for k in range(3):
        W.make_pulse(sd_seq[k])
        W.advance_time(pop, 0, sd_seq[k])
    ct_s, ct_p, ct_a = timed_steps(torch, W, pop, sd_seq, csteps, flush=flush)
    comp = {"pulses_per_s": csteps / (sum(ct_s) / 1000.0), "step_ms": statistics.mean(ct_s),
            "pulse_ms": statistics.mean(ct_p), "advance_ms": statistics.mean(ct_a), "steps": csteps}
    W.close()
    del flush
    torch.cuda.empty_cache()

    extras = {}
    if world == 1:
        wanted = [s for s in args.sections.split(",") if s in SECTIONS]
        if "precision" in wanted:
            extras["precision"] = bench_precision(torch, rsc, synth, dev, steps=min(args.steps, 50))
        if "batch" in wanted:
            extras["batch"] = bench_batch(torch, rsc, synth, dev, steps=500)
        if "les" in wanted:
            extras["les"] = bench_les(torch, rsc, synth, dev, S)
        if "large" in wanted:
            extras["large"] = bench_large(torch, rsc, synth, dev, chunks=100)
        if "small" in wanted and not args.no_cpu_baseline:
            extras["small"] = bench_small(torch, rsc, synth, dev)

    # CPU baseline: the oracle on a bounded sample of the same workload
    cpu = None
    if not args.no_cpu_baseline:
        cpu_value, cores = cpu_reference(S, pulses=12, warm=1)
        cpu = {"value": cpu_value, "unit": UNIT, "cores": cores, "kind": "port", "cpu": cpu_model(),
               "sample": "12 full-size pulses (make_pulse + advance_time) after 1 warm, OpenMP on all host cores"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded LES/ADM/RCS tables, see simradar_gb300/synth.py)",
        "config": workload_config(N_RAIN),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 64, "d2h_bytes_per_step": G * 16,
                "blocking_read_value": e2e_blocking},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "clocks": clk,
        "gpu_launches": int(launches),
        "scatterer_updates_per_s": value * S.num_scats,
        "kernel_ms": {"k_pulse_group<0, 2, 1>": pul_ms, "advance (k_advance_rain + k_advance_debris)": adv_ms,
                      "note": "the pulse and the advance of a step run concurrently on two streams; each is "
                              "timed on its own stream, the step from its start to both ends"},
        "compensated": comp,
        "sort": {"interval_steps": interval, "ms_per_sort": sort_ms, "amortized_ms_per_step": sort_ms / interval,
                 "sorts_in_value_window": int(sorts_value), "sorts_in_e2e_window": int(sorts_e2e),
                 "note": "value and e2e include the spatial sort at its amortised cost (ms_per_sort / "
                         "interval per step): the sorts that fell in each window are replaced by "
                         "steps / interval of them"},
    }
    line.update(extras)
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sections", default=",".join(SECTIONS),
                    help="extra one-GPU sections to run (comma list of %s; '' for none)" % ", ".join(SECTIONS))
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
