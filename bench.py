"""Benchmark: correlated Gsamples/s of the FX correlator on one GB300.

Workload (one "step"): the 256-station dual-polarisation configuration --
512 inputs of 2-bit offset-binary samples (rho = 0.02 common signal),
2048-point real FFTs (1024 channels), 4096 spectra integrated, i.e.
8,388,608 samples per input and 4.29 G samples per step, correlated into all
131,328 lower-triangle products x 1024 channels.  A step runs unpack + FFT +
X stage through the engine's C ABI.

* value : device-resident inputs and outputs (cellspe_fx_correlate with
          CELLSPE_MEM_DEVICE), K steps bracketed by synchronize + CUDA events.
* e2e   : the same job with pinned HOST buffers: every step copies the 2-bit
          input to the GPU and the visibilities back.  Measured through the
          correlation service (two jobs in flight, so one job's copies overlap
          the other's stages), and as one blocking call per step ("sync").
* roofline: the dominant kernel's algorithmic rate, from CUDA events the
          library records on its own stream around each stage.
* error : after the timed regions, the timed job's visibilities against the
          FP64 oracle on a seeded subset of inputs x channels with the full K
          (amplitude and phase error; the oracle is only the checker), and the
          tensor-core path against the FP32 path over every product.
* cpu_baseline: the FX path of the CPU oracle (restated genericAddProduct_32fc_conj
          X stage, radix-2 FFT standing in for the absent FFTW) on a bounded
          sample of the same inputs, all host threads.

Under torchrun each rank runs its own job (a different subband) on its own
GPU: weak scaling, no data-path collective.  ``--impl reference`` times the
CPU implementation alone.
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
sys.path.insert(0, str(ROOT / "cellspe-tasklib_gb300"))
sys.path.insert(0, str(ROOT))

S, N, K = 512, 2048, 4096          # 256 stations x 2 pols, 2048-pt FFT, 4096 spectra
RHO = 0.02
C = N // 2
P = S * (S + 1) // 2
T = N * K


def _peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text()), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index, self.rows, self.proc = index, [], None
        self.t0, self.t1 = None, None

    def mark_start(self):
        self.t0 = time.monotonic()

    def mark_end(self):
        self.t1 = time.monotonic()

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.monotonic(), [x.strip() for x in line.split(",")]))

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        """Samples taken between mark_start and mark_end (the timed region)."""
        rows = [r for t, r in self.rows
                if (self.t0 is None or t >= self.t0) and (self.t1 is None or t <= self.t1)]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if len(r) > 3 + i and r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(raw_host: np.ndarray, k_sample: int, nthreads: int):
    import oracle

    sample = np.ascontiguousarray(raw_host[:, : k_sample * N // 4])
    t0 = time.perf_counter()
    oracle.fx_fp32(sample, S, N, k_sample, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return S * k_sample * N / dt / 1e9, dt


def _serving_jobs(rng, seconds: float, rate: float):
    s_choices, c_choices = [4, 8, 24, 64, 200], [256, 1024, 4096, 16384]
    t_arr, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate) if rate > 0 else 0.0
        if t > seconds or (rate <= 0 and len(t_arr) >= int(seconds)):
            break
        t_arr.append(t)
    jobs = [(int(rng.choice(s_choices)), int(rng.choice(c_choices)), 2 ** int(rng.integers(18, 25))) for _ in t_arr]
    return jobs, t_arr


def _serve(cg, torch, jobs, t_arr, x_mode, raw_pool, keep=(), batch_inputs=0):
    """Submit the jobs at their arrival times (all at once when t_arr is all 0),
    at most 64 outstanding; returns latencies, makespan, stats and the kept outputs."""
    svc = cg.Service(batch_inputs=batch_inputs)
    pending, lat, kept = [], [], {}
    t0 = time.perf_counter()
    for n, ((S, C, T), ta) in enumerate(zip(jobs, t_arr)):
        now = time.perf_counter() - t0
        if ta > now:
            time.sleep(ta - now)
        raw = raw_pool[: S * T // 4].view(S, T // 4)
        vis = torch.empty((C, S * (S + 1) // 2), dtype=torch.complex64, device="cuda")
        p = cg.fx_params(S, 2 * C, T // (2 * C), T // 4, x_mode=x_mode)
        pending.append((svc.submit(p, raw, vis), vis, n))
        while len(pending) > 64:                      # bounded outstanding outputs
            jid, v, k = pending.pop(0)
            lat.append(svc.wait(jid))
            if k in keep:
                kept[k] = v
    for jid, v, k in pending:
        lat.append(svc.wait(jid))
        if k in keep:
            kept[k] = v
    makespan = time.perf_counter() - t0
    st = svc.stats()
    svc.close()
    return lat, makespan, st, kept


def run_serving(cg, torch, seconds: float, rate: float, x_mode: int, seed: int = 5, error_jobs: int = 16,
                near_seconds: float = 10.0):
    """Batched streaming service: Poisson arrivals, uneven jobs (S, C, T) as in the
    serving configuration, device-resident buffers; latency is submit -> done.
    The service runs with its defaults: two streams, jobs under 2^24 samples on
    a high-priority stream.  Three runs of the same job mix:
      * the Poisson window at `rate` jobs/s;
      * capacity: 2000 jobs submitted at once (64 outstanding), served rate;
      * near capacity: Poisson arrivals at 0.8 x the capacity job rate for
        `near_seconds`;
    and, for `error_jobs` seeded jobs of the first run, the tensor-core result
    against the FP32 CUDA-core path (max over products of the relative L2
    error over channels)."""
    rng = np.random.default_rng(seed)
    jobs, t_arr = _serving_jobs(rng, seconds, rate)
    max_raw = 200 * (1 << 24) // 4                   # the mix's largest job (S = 200, T = 2^24)
    g = torch.Generator(device="cuda").manual_seed(seed)
    raw_pool = torch.randint(0, 256, (max_raw,), dtype=torch.uint8, device="cuda", generator=g)
    # outputs of up to 256 MB are kept for the error check
    small = [k for k, (S, C, T) in enumerate(jobs) if C * S * (S + 1) // 2 * 8 <= 256 << 20]
    keep = set(np.random.default_rng(seed + 1).choice(small, size=min(error_jobs, len(small)), replace=False).tolist())
    lat, makespan, st, kept = _serve(cg, torch, jobs, t_arr, x_mode, raw_pool, keep)
    samples = sum(S * T for S, _, T in jobs)
    res = {"jobs": len(jobs), "arrival_rate_per_s": rate, "window_s": seconds,
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "offered_gsamples_s": samples / seconds / 1e9, "served_gsamples_s": samples / makespan / 1e9,
           "max_concurrent_jobs": st["max_running"], "failed": st["failed"],
           "batched_jobs": st["batched_jobs"], "batched_launches": st["batched_launches"],
           "p99_queue_ms": st["p99_queue_ms"], "streams": 2, "priority_samples": 1 << 24,
           "job_mix": "S in {4,8,24,64,200}, C in {256,1024,4096,16384}, T = 2^U, U in [18,24]"}
    if x_mode == cg.X_TC_FP16 and kept:
        errs = []
        for k, v in kept.items():
            S, C, T = jobs[k]
            ref = torch.empty_like(v)
            raw = raw_pool[: S * T // 4].view(S, T // 4)
            cg.fx_correlate(cg.fx_params(S, 2 * C, T // (2 * C), T // 4, x_mode=cg.X_FP32), raw, ref)
            num = torch.linalg.vector_norm(v - ref, dim=0)
            errs.append(float((num / torch.linalg.vector_norm(ref, dim=0)).max()))
        res["tc_vs_fp32"] = {"jobs": len(errs), "max_rel": max(errs), "median_rel": float(np.median(errs)),
                             "sample": "seeded jobs with outputs up to 256 MB; max over products of the "
                                       "relative L2 error over channels"}
    kept.clear()
    # capacity: the same mix, all submitted at once
    cj, _ = _serving_jobs(np.random.default_rng(seed + 2), 2000, 0.0)
    clat, cspan, cst, _ = _serve(cg, torch, cj, [0.0] * len(cj), x_mode, raw_pool)
    csamples = sum(S * T for S, _, T in cj)
    cap_rate = len(cj) / cspan
    res["capacity"] = {"jobs": len(cj), "served_gsamples_s": csamples / cspan / 1e9, "jobs_per_s": cap_rate,
                       "failed": cst["failed"], "max_concurrent_jobs": cst["max_running"],
                       "batched_jobs": cst["batched_jobs"], "batched_launches": cst["batched_launches"]}
    if near_seconds > 0:
        nrate = 0.8 * cap_rate
        nj, nt = _serving_jobs(np.random.default_rng(seed + 3), near_seconds, nrate)
        nsamples = sum(S * T for S, _, T in nj)
        # the same arrivals with the service's default batching and with batching off
        for key, b in (("near_capacity", 0), ("near_capacity_unbatched", -1)):
            nlat, nspan, nst, _ = _serve(cg, torch, nj, nt, x_mode, raw_pool, batch_inputs=b)
            res[key] = {"jobs": len(nj), "arrival_rate_per_s": nrate, "window_s": near_seconds,
                        "offered_gsamples_s": nsamples / near_seconds / 1e9,
                        "served_gsamples_s": nsamples / nspan / 1e9,
                        "p50_ms": float(np.percentile(nlat, 50)), "p99_ms": float(np.percentile(nlat, 99)),
                        "p99_queue_ms": nst["p99_queue_ms"], "failed": nst["failed"],
                        "max_concurrent_jobs": nst["max_running"], "batched_jobs": nst["batched_jobs"],
                        "batched_launches": nst["batched_launches"]}
    del raw_pool
    return res


def _time_calls(torch, fn, steps: int, warmup: int) -> float:
    """Milliseconds per call by CUDA events (device-resident buffers)."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1) / steps


def vis_error(torch, raw, vis, Sx: int, Nx: int, Kx: int, n_inputs: int, n_chans: int, seed: int,
              start_sample: int = 0, delay=None):
    """Amplitude and phase error of channel-major visibilities [C][P] against the
    FP64 oracle on a seeded subset of inputs x channels with the full K (the
    accuracy check after the timed region; the oracle is the checker here).
    delay = (shift, phase0, dphase) from the FP64 delay model, or None."""
    import oracle

    rng = np.random.default_rng(seed)
    inputs = sorted(int(i) for i in rng.choice(Sx, size=n_inputs, replace=False))
    chans = sorted(int(c) for c in rng.choice(Nx // 2, size=n_chans, replace=False))
    sh, p0, dp = (None, None, None) if delay is None else (d[inputs] for d in delay)
    t0 = time.perf_counter()
    ref, autos = oracle.fx_vis_subset_f64(raw[inputs].cpu().numpy(), Nx, Kx, chans, start_sample, sh, p0, dp)
    n = len(inputs)
    pidx = [inputs[a] * (inputs[a] + 1) // 2 + inputs[b] for a in range(n) for b in range(a + 1)]
    sel = vis[torch.as_tensor(chans, device=vis.device)][:, torch.as_tensor(pidx, device=vis.device)].cpu().numpy()
    got = np.zeros((n, n, len(chans)), np.complex128)
    q = 0
    for a in range(n):
        for b in range(a + 1):
            got[a, b] = sel[:, q]
            q += 1
    err = oracle.vis_errors(got, ref, autos, Kx)
    err.update({"subset": f"{n} inputs ({n * (n + 1) // 2} products) x {len(chans)} channels, full K={Kx}",
                "reference": "FP64 oracle", "oracle_s": round(time.perf_counter() - t0, 1)})
    return err


def rel_all(torch, v, ref) -> float:
    """Max over products (columns of [C][P]) of ||v - ref|| / ||ref|| over channels."""
    num = torch.linalg.vector_norm(v - ref, dim=0)
    den = torch.linalg.vector_norm(ref, dim=0)
    return float((num / den).max())


def run_configs(cg, torch, x_mode: int, with_cpu: bool, raw, vis_main):
    """The other benchmark configurations, measured beside the headline: the FP32
    path on the headline job (same input; its error, and the tensor-core path's
    error against it), the Mark5B spectrometer (payload and framed recordings)
    and the 16-station delay-tracked job, each with its CPU rate and error."""
    out = {}
    # -- FP32 CUDA-core path on the headline job (tensor-core vs FP32 ratio)
    T = N * K
    g = torch.Generator(device="cuda").manual_seed(4)
    vis = torch.empty((C, P), dtype=torch.complex64, device="cuda")
    p32 = cg.fx_params(S, N, K, T // 4, x_mode=cg.X_FP32, vis_order=cg.VIS_CHANNEL_MAJOR)
    ms = _time_calls(torch, lambda: cg.fx_correlate(p32, raw, vis), steps=3, warmup=1)
    out["fp32_path"] = {"value": S * T / (ms * 1e-3) / 1e9, "unit": "Gsamples/s", "ms_per_step": ms,
                        "workload": "same job and input as the headline, x_mode = FP32 CUDA cores",
                        "error": vis_error(torch, raw, vis, S, N, K, 16, 32, seed=K)}
    if x_mode == cg.X_TC_FP16:
        out["tc_vs_fp32_max_rel"] = rel_all(torch, vis_main, vis)
    # -- the same job with the INT8 X stage (mma.sync IMMA; tcgen05 has no kind::i8 on sm_103a)
    vis8 = torch.empty((C, P), dtype=torch.complex64, device="cuda")
    p8 = cg.fx_params(S, N, K, T // 4, x_mode=cg.X_INT8, vis_order=cg.VIS_CHANNEL_MAJOR)
    ms8 = _time_calls(torch, lambda: cg.fx_correlate(p8, raw, vis8), steps=3, warmup=1)
    st8 = cg.stage_times()
    x8_ops = 8.0 * C * P * K                                  # 4 real int8 MACs per complex MAC
    out["int8_path"] = {"value": S * T / (ms8 * 1e-3) / 1e9, "unit": "Gsamples/s", "ms_per_step": ms8,
                        "workload": "same job and input as the headline, x_mode = INT8 (per input/channel "
                                    "max-abs int8 spectra, mma.sync m16n8k32 IMMA, int32 sums)",
                        "stages_ms": {"f_stage_and_quantise": st8[1], "x_stage": st8[2]},
                        "x_stage_tops": x8_ops / (st8[2] * 1e-3) / 1e12,
                        "imma_peak_tops": 151.0,     # register-only mma.sync s8 m16n8k32 loop on this GB300
                        "error": vis_error(torch, raw, vis8, S, N, K, 16, 32, seed=K),
                        "int8_vs_fp32_max_rel": rel_all(torch, vis, vis8)}
    del vis, vis8

    import synth

    # -- Mark5B spectrometer: 16 subbands x 2^25 samples, N = 65536, overlap 2, cosine^2, PCal
    nsub, nsamp, NS, fs = 16, 1 << 25, 65536, 32e6
    kspec = nsamp // NS
    payload = torch.randint(0, 256, (nsamp * nsub // 4,), dtype=torch.uint8, device="cuda", generator=g)
    power = torch.empty((nsub, 1, NS // 2 + 1), dtype=torch.float32, device="cuda")
    bins = torch.empty((nsub, 1, 32), dtype=torch.complex64, device="cuda")
    sp = cg.spec_params(NS, 2, 2, kspec, 1, nsub, payload.numel(), tonebins=32, rotatorlen=32, ntones=16,
                        fs_hz=fs, memory=cg.MEM_DEVICE)
    ms = _time_calls(torch, lambda: cg.spectrometer(sp, payload, power, bins), steps=5, warmup=2)
    nffts = nsub * (2 * kspec - 1)
    res = {"value": nsub * nsamp / (ms * 1e-3) / 1e9, "unit": "Gsamples/s", "ms_per_step": ms,
           "fft_tflops": nffts * 2.5 * NS * 16 / (ms * 1e-3) / 1e12,
           "workload": "Mark5B 16 subbands x 2^25 samples (1 s at 32 MS/s), N=65536, overlap 2, cosine^2, PCal 32 bins"}
    # framed recording: 16-byte headers per 10000-byte payload, blanking on
    nf = -(-payload.numel() // 10000)
    framed = torch.zeros((nf, 10016), dtype=torch.uint8, device="cuda")
    framed[:, 0:4] = torch.tensor([0xED, 0xDE, 0xAD, 0xAB], dtype=torch.uint8, device="cuda")
    flat = framed[:, 16:].reshape(-1)
    flat[: payload.numel()] = payload
    framed = framed.reshape(-1)
    spf = cg.spec_params(NS, 2, 2, kspec, 1, nsub, framed.numel(), layout=cg.SPEC_MARK5B_FRAMED, tonebins=32,
                         rotatorlen=32, ntones=16, fs_hz=fs, memory=cg.MEM_DEVICE)
    ms_f = _time_calls(torch, lambda: cg.spectrometer(spf, framed, power, bins), steps=5, warmup=2)
    res["framed_value"] = nsub * nsamp / (ms_f * 1e-3) / 1e9
    res["framed_ms_per_step"] = ms_f
    del framed
    # the same samples as a VDIF recording: 32-byte headers per 8000-byte payload
    # (1024 Mbps, 16000 frames per second), every frame validated on the device
    nfv = -(-payload.numel() // 8000)
    mbps = int(fs * 2 * nsub / 1e6)
    hdr = synth.vdif_frames(np.zeros(nfv * 8000, np.uint8), 8000, nsub, mbps).reshape(nfv, 8032)[:, :32]
    vdif = torch.zeros((nfv, 8032), dtype=torch.uint8, device="cuda")
    vdif[:, :32] = torch.from_numpy(hdr).cuda()
    vflat = vdif[:, 32:].reshape(-1)
    vflat[: payload.numel()] = payload
    vdif = vdif.reshape(-1)
    spv = cg.spec_params(NS, 2, 2, kspec, 1, nsub, vdif.numel(), layout=cg.SPEC_VDIF_FRAMED, levels=cg.LEVELS_VDIF,
                         tonebins=32, rotatorlen=32, ntones=16, fs_hz=fs, memory=cg.MEM_DEVICE)
    ms_v = _time_calls(torch, lambda: cg.spectrometer(spv, vdif, power, bins), steps=5, warmup=2)
    res["vdif_value"] = nsub * nsamp / (ms_v * 1e-3) / 1e9
    res["vdif_ms_per_step"] = ms_v
    del vdif
    if with_cpu:
        import oracle

        # oracle spectrometer (single thread) on one subband, 16 FFT lengths
        x = np.random.default_rng(2).standard_normal(16 * NS).astype(np.float32)
        t0 = time.perf_counter()
        oracle.spectrometer(x, NS, 2, 2, 16, 32, 32, 0.0, fs)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": x.size / dt / 1e9, "unit": "Gsamples/s", "cores": 1, "kind": "port",
                               "sample": f"1 subband x {16 * NS} samples, {dt:.2f} s"}
    out["mark5b_spectrometer"] = res
    del payload, power, bins

    # -- 16-station dual-pol (32 inputs), N = 8192, K = 4096, cubic delay model, one subband
    S3, N3, K3 = 32, 8192, 4096
    T3 = N3 * K3
    fs3, lo3, rho3 = 32e6, 8.4e9, 0.3
    margin = 1 << 17
    rng = np.random.default_rng(3)
    poly = np.zeros((S3, 4))
    poly[:, 0] = rng.uniform(-2e-3, 2e-3, S3)
    poly[:, 1] = rng.uniform(-3e-6, 3e-6, S3)
    poly[:, 2] = rng.uniform(-1e-9, 1e-9, S3)
    poly[:, 3] = rng.uniform(-1e-12, 1e-12, S3)
    raw3 = synth.device_delayed_stations(S3, N3, K3, poly, fs3, lo3, rho3, seed=33, margin=margin)
    dpoly = torch.from_numpy(poly).cuda()
    vis3 = torch.empty((N3 // 2, S3 * (S3 + 1) // 2), dtype=torch.complex64, device="cuda")
    r3 = {"workload": "32 inputs, N=8192 (4096 channels), K=4096, cubic delay per input (a0 within +-2 ms, "
                      "a1 within +-3 us/s), fs 32 MS/s, LO 8.4 GHz, one of 8 subbands; a sky signal (rho 0.3) "
                      "delayed by the same model, so delay-corrected cross products are coherent"}
    import oracle

    delay = oracle.delay_state_f64(poly, N3, K3, fs3, lo3)
    outs = {}
    for name, mode in (("tc", cg.X_TC_FP16), ("fp32", cg.X_FP32)):
        p3 = cg.fx_params(S3, N3, K3, raw3.shape[1], x_mode=mode, vis_order=cg.VIS_CHANNEL_MAJOR,
                          start_sample=margin, fs_hz=fs3, lo_hz=lo3)
        ms3 = _time_calls(torch, lambda: cg.fx_correlate(p3, raw3, vis3, delay_poly=dpoly), steps=3, warmup=1)
        r3[name] = {"value": S3 * T3 / (ms3 * 1e-3) / 1e9, "unit": "Gsamples/s", "ms_per_step": ms3,
                    "error": vis_error(torch, raw3, vis3, S3, N3, K3, 8, 32, seed=16, start_sample=margin,
                                       delay=delay)}
        outs[name] = vis3.clone()
    r3["tc_vs_fp32_max_rel"] = rel_all(torch, outs["tc"], outs["fp32"])
    out["fx_16station_delay"] = r3
    del raw3, vis3, outs
    torch.cuda.empty_cache()
    return out


def run_reference(args):
    """CPU implementation of the path (the oracle's FX restatement), all host threads."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import synth

    nthreads = os.cpu_count() or 1
    k_sample = args.cpu_segments
    raw = synth.stations_offset_binary(S, k_sample * N, rho=RHO, seed=4)
    for _ in range(args.warmup):
        cpu_baseline(raw, max(1, k_sample // 8), nthreads)
    vals, secs = [], []
    for _ in range(args.steps):
        v, dt = cpu_baseline(raw, k_sample, nthreads)
        vals.append(v)
        secs.append(dt)
    value = statistics.median(vals)
    sample = f"{S} inputs x {k_sample} segments x {N} samples ({S * k_sample * N / 1e6:.0f} M samples) per step"
    line = {
        "metric": "correlated Gsamples/s", "value": value, "unit": "Gsamples/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * statistics.median(secs), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded 2-bit offset binary, rho=0.02)",
        "config": {"workload": "256-station dual-pol FX: S=512, N=2048, C=1024, K=4096", "inputs": S,
                   "fft_points": N, "segments": K},
        "cpu_baseline": {"value": value, "unit": "Gsamples/s", "cores": nthreads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "Gsamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="tc", choices=["tc", "fp32"])
    ap.add_argument("--e2e-steps", type=int, default=10,
                    help="timed end-to-end calls (their mean: single calls over the CPU-GPU link vary by a few ms)")
    ap.add_argument("--cpu-segments", type=int, default=64,
                    help="segments per step of the reference arm (--impl reference)")
    ap.add_argument("--cpu-baseline-segments", type=int, default=1024,
                    help="segments of this arm's cpu_baseline sample (~11 s on 16 cores; 1 core: 1/16 of it)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-error", action="store_true", help="skip the FP64 accuracy check of the timed job")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the FP32-path, spectrometer and delay-tracked measurements")
    ap.add_argument("--serve-seconds", type=float, default=30.0,
                    help="length of the Poisson arrival window of the serving measurement (0 skips it)")
    ap.add_argument("--segments", type=int, default=K,
                    help="spectra per integration (smaller values make a profiling-sized case)")
    ap.add_argument("--inputs", type=int, default=S,
                    help="inputs (smaller values make a profiling-sized case)")
    ap.add_argument("--fft-points", type=int, default=N,
                    help="FFT length (smaller values make a profiling-sized case with fewer channels)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch

    import cellspe_gpu as cg
    import replicas
    import synth

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    x_mode = cg.X_TC_FP16 if args.mode == "tc" else cg.X_FP32
    S_run, K_run = args.inputs, args.segments
    P_run = S_run * (S_run + 1) // 2
    N_run = args.fft_points
    C_run = N_run // 2
    T_run = N_run * K_run
    raw = synth.device_stations(S_run, T_run, RHO, seed=replicas.job_seed(rank))
    vis = torch.empty((C_run, P_run), dtype=torch.complex64, device="cuda")
    params = cg.fx_params(S_run, N_run, K_run, T_run // 4, x_mode=x_mode, vis_order=cg.VIS_CHANNEL_MAJOR)
    clk = ClockSampler(local).__enter__()             # running before the timed region
    for _ in range(args.warmup):
        cg.fx_correlate(params, raw, vis)

    # ---- device-resident timed region ------------------------------------
    stage_sum = np.zeros(4)
    barrier()
    l0 = cg.kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk.mark_start()
    e0.record()
    for _ in range(args.steps):
        cg.fx_correlate(params, raw, vis)
        stage_sum += np.array(cg.stage_times())
    torch.cuda.synchronize()
    e1.record()
    e1.synchronize()
    clk.mark_end()
    clk.__exit__(None, None, None)
    launches = cg.kernel_launches() - l0
    ms = replicas.max_over_ranks(e0.elapsed_time(e1), dist, device="cuda")
    ms_step = ms / args.steps
    value = replicas.aggregate_gsamples(world, S_run * T_run, ms_step)
    stage_ms = stage_sum / args.steps

    # ---- end to end through the C ABI with host buffers --------------------
    raw_h = np.empty((S_run, T_run // 4), np.uint8)
    raw_h[:] = raw.cpu().numpy()
    e2e_ms, e2e_value, e2e_sync, e2e_concurrent = None, None, None, None
    if not args.no_e2e:
        pin_raw = torch.from_numpy(raw_h).pin_memory()
        pin_vis = [torch.empty((C_run, P_run), dtype=torch.complex64).pin_memory() for _ in range(2)]
        raw_np, vis_np = pin_raw.numpy(), [v.numpy() for v in pin_vis]
        hparams = cg.fx_params(S_run, N_run, K_run, T_run // 4, x_mode=x_mode, vis_order=cg.VIS_CHANNEL_MAJOR)
        # (a) one blocking cellspe_fx_correlate call at a time: the input copy,
        # both stages and the visibility copy of a job in series (the input and
        # output copies overlap the stages within the job)
        for _ in range(max(1, args.warmup)):         # the first call sizes the workspace
            cg.fx_correlate(hparams, raw_np, vis_np[0])
        barrier()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record()
        for _ in range(args.e2e_steps):
            cg.fx_correlate(hparams, raw_np, vis_np[0])
        torch.cuda.synchronize()
        f1.record()
        f1.synchronize()
        sync_ms = replicas.max_over_ranks(f0.elapsed_time(f1) / args.e2e_steps, dist, device="cuda")
        e2e_sync = {"value": replicas.aggregate_gsamples(world, S_run * T_run, sync_ms), "ms_per_step": sync_ms,
                    "mode": "one blocking cellspe_fx_correlate call per step"}
        cg.lib().cellspe_release_workspace()
        # (b) the same jobs through the correlation service (cellspe_service_*,
        # two streams, host buffers): step i+1's input copy and F stage run
        # while step i's X stage and visibility copy finish; every step still
        # copies its 1.07 GB of samples in and its 1.08 GB of visibilities out.
        svc = cg.Service(max_streams=2, priority_samples=-1)
        jobs = [cg.fx_params(S_run, N_run, K_run, T_run // 4, x_mode=x_mode, vis_order=cg.VIS_CHANNEL_MAJOR)
                for _ in range(2)]
        # warm-up with two jobs in flight, so that both workers have sized
        # their workspaces (jobs waited one at a time can all land on one
        # worker, and the other's first allocation then falls in the timed loop)
        for _ in range(max(2, args.warmup)):
            warm = [svc.submit(jobs[w], raw_np, vis_np[w]) for w in range(2)]
            for jid in warm:
                svc.wait(jid)
        barrier()
        pending = []
        t_e2e = time.perf_counter()
        for i in range(args.e2e_steps):
            if len(pending) == 2:
                svc.wait(pending.pop(0))
            pending.append(svc.submit(jobs[i % 2], raw_np, vis_np[i % 2]))
        for jid in pending:
            svc.wait(jid)
        torch.cuda.synchronize()
        e2e_ms = replicas.max_over_ranks(1e3 * (time.perf_counter() - t_e2e) / args.e2e_steps, dist, device="cuda")
        e2e_value = replicas.aggregate_gsamples(world, S_run * T_run, e2e_ms)
        e2e_concurrent = svc.stats()["max_running"]
        svc.close()
        del pin_vis, pin_raw

    # ---- roofline of the dominant kernel -----------------------------------
    # DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) measured by
    # ncu on cases larger than L2 with the same per-unit work, scaled by the
    # units one launch here processes: the warp-FFT F stage moved 4,375 B per
    # input-segment (512 inputs x 512 segments, N = 2048, k-blocked FP16
    # spectra, --set full); the warp-specialised tensor-core F stage 4,578 B
    # and the tensor-core X stage 2,074 B per (channel, segment) read plus
    # 1.025 MB of visibilities written per channel (512 inputs x 4096
    # segments, channel-grouped spectra, one-pass dram__bytes_read/write
    # capture).  None where no capture of that kernel exists.
    F_TRAFFIC_PER_SEGMENT = {"k_fx_fstage_w2048": 4375.0, "k_fx_fstage_tc32ws": 4578.0}
    X_TRAFFIC_PER_CHANNEL = 2074.0 * K_run + 1.025e6
    peaks, peak_kind = _peaks()
    f_ms, x_ms = stage_ms[1], stage_ms[2]
    f_bytes = S_run * K_run * (N_run // 4 + C_run * (8 if x_mode == cg.X_FP32 else 4))     # raw in + spectra out
    x_flops = 8.0 * P_run * C_run * K_run                                              # 8 real flops per CMAC, triangle
    stages = {"f_stage_ms": f_ms, "x_stage_ms": x_ms, "output_ms": stage_ms[3],
              "f_stage_gbs": f_bytes / (f_ms * 1e-3) / 1e9,
              "x_stage_tflops": x_flops / (x_ms * 1e-3) / 1e12}
    if x_ms >= f_ms:
        if x_mode == cg.X_FP32:
            fp32_peak = 152 * 128 * 2 * (peaks.get("sm_max_mhz", 2070.0) * 1e6) / 1e12
            roof = {"bound": "fp32", "kernel": "k_xmac_f32", "achieved": stages["x_stage_tflops"],
                    "peak": fp32_peak, "unit": "TFLOP/s", "frac": stages["x_stage_tflops"] / fp32_peak,
                    "peak_source": "nominal FP32 CUDA-core rate 152 SM x 128 FMA x 2 x max clock",
                    "traffic": None}
        else:
            pk = peaks["bf16_tflops"]
            roof = {"bound": "tensor", "kernel": "k_xmac_tc", "achieved": stages["x_stage_tflops"], "peak": pk,
                    "unit": "TFLOP/s", "frac": stages["x_stage_tflops"] / pk,
                    "peak_source": f"{peak_kind} dense bf16 (burst)",
                    "traffic": X_TRAFFIC_PER_CHANNEL * C_run}
    else:
        pk = peaks["hbm_gbs"]
        # the F-stage kernel the library picks for this job (fstage.cu's dispatch)
        tc_f = x_mode == cg.X_TC_FP16 and N_run == 2048 and os.environ.get("CELLSPE_FSTAGE_TC") == "1"
        tc32 = os.environ.get("CELLSPE_FSTAGE_TC32", "2")[:1] or "2"
        if x_mode == cg.X_TC_FP16 and N_run == 2048 and K_run % 32 == 0 and tc32 in "12":
            fk = "k_fx_fstage_tc32ws" if tc32 == "2" else "k_fx_fstage_tc32"
        elif tc_f:
            fk = "k_fx_fstage_tc"
        else:
            fk = ("k_fx_fstage_w2048" if N_run == 2048 else "k_fx_fstage_wbig" if N_run >= 4096 else "k_fx_fstage")
        per_seg = F_TRAFFIC_PER_SEGMENT.get(fk)
        roof = {"bound": "hbm", "kernel": fk, "achieved": stages["f_stage_gbs"], "peak": pk,
                "unit": "GB/s", "frac": stages["f_stage_gbs"] / pk, "peak_source": f"{peak_kind} HBM copy",
                "traffic": per_seg * S_run * K_run if per_seg else None,
                "note": ("F stage is bound by the LSU data pipe (shared memory + spectra stores, 67% busy) and "
                         "its epilogue warps (ncu), not HBM bandwidth; DRAM bytes equal the algorithmic ones"
                         if fk == "k_fx_fstage_tc32ws" else
                         "F stage is bound by instruction issue and the shared-memory pipe (ncu), not HBM")}

    # ---- accuracy of the timed job (after the timed regions) ----------------
    # FP64 oracle on a seeded subset (16 inputs x 32 channels, full K) of this
    # very run's visibilities; at rho = 0.02 the cross products sit below the
    # 3-sigma noise floor, so the phase bar is also checked on the same shape at
    # rho = 0.3 with K = 1024, where they rise above it.
    error = None
    if not args.no_error:
        error = vis_error(torch, raw, vis, S_run, N_run, K_run, min(16, S_run), min(32, C_run), seed=K_run)
        if S_run == S and N_run == N:
            k_ph = min(K_run, 1024)
            raw_ph = synth.device_stations(S_run, N_run * k_ph, 0.3, seed=40 + rank)
            vis_ph = torch.empty((C_run, P_run), dtype=torch.complex64, device="cuda")
            cg.fx_correlate(cg.fx_params(S_run, N_run, k_ph, raw_ph.shape[1], x_mode=x_mode,
                                         vis_order=cg.VIS_CHANNEL_MAJOR), raw_ph, vis_ph)
            ph = vis_error(torch, raw_ph, vis_ph, S_run, N_run, k_ph, 16, 32, seed=k_ph)
            error["phase_check_rho0.3"] = {k: ph[k] for k in ("max_rel_amp", "max_phase_deg", "phase_cells",
                                                               "cross_products_above_floor", "cross_products")}
            error["phase_check_rho0.3"]["job"] = f"S={S_run}, N={N_run}, K={k_ph}, rho=0.3"
            del raw_ph, vis_ph
        error["bars"] = ("tensor-core: <= 1e-3 relative amplitude per product, <= 0.05 deg above the noise floor; "
                         "FP32: <= 1e-5")

    serving = None
    if args.serve_seconds > 0:
        serving = run_serving(cg, torch, args.serve_seconds, 200.0, x_mode)
    configs = None
    if not args.no_configs and N_run == N and S_run == S:
        configs = run_configs(cg, torch, x_mode, (rank == 0 and not args.no_cpu), raw, vis)

    cpu = None
    if rank == 0 and not args.no_cpu:
        nthreads = os.cpu_count() or 1
        kb = min(args.cpu_baseline_segments, K_run)
        v, dt = cpu_baseline(raw_h, kb, nthreads)
        v1, dt1 = cpu_baseline(raw_h, max(1, kb // 16), 1)
        cpu = {"value": v, "unit": "Gsamples/s", "cores": nthreads, "kind": "port",
               "sample": f"{S_run} inputs x {kb} segments x {N_run} samples, {dt:.1f} s",
               "value_1core": v1,
               "sample_1core": f"{S_run} inputs x {max(1, kb // 16)} segments, {dt1:.1f} s"}

    if rank == 0:
        line = {
            "metric": "correlated Gsamples/s", "value": value, "unit": "Gsamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f16-tc/f32-acc" if x_mode == cg.X_TC_FP16 else "f32",
            "data": "synthetic (seeded 2-bit offset binary, rho=0.02, generated on device)",
            "config": {"workload": (f"256-station dual-pol FX: S=512, N={N_run}, C={C_run}, K={K_run}" if S_run == S
                                    else f"FX: S={S_run}, N={N_run}, C={C_run}, K={K_run}"),
                       "inputs": S_run, "fft_points": N_run, "channels": C_run, "segments": K_run, "products": P_run,
                       "x_mode": args.mode, "vis_order": "channel-major [C][P]",
                       "l2": "inputs larger than L2 (1.07 GB raw, spectra 8.6/17 GB, vis 1.07 GB)",
                       "parallelism": f"replicas x{world} (one job per GPU)"},
            "e2e": {"value": e2e_value, "unit": "Gsamples/s", "h2d_bytes_per_step": int(S_run * T_run // 4),
                    "d2h_bytes_per_step": int(C_run * P_run * 8), "ms_per_step": e2e_ms,
                    "mode": "host buffers through cellspe_service_* (two streams, two jobs in flight; "
                            "wall clock over e2e_steps jobs)",
                    "max_concurrent_jobs": e2e_concurrent, "sync": e2e_sync},
            "gpu_launches": int(launches),
            "roofline": roof,
            "error": error,
            "stages": stages,
            "clocks": clk.summary(),
            "serving": serving,
            "configs": configs,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
