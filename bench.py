#!/usr/bin/env python3
"""SENSE-CG iterations/s on one GB300 (gridFFT E^H W E + FP64-scalar CG).

Workload: 256^3 image, 32 coils, 3D radial 65536 x 256 (16.8M samples per coil),
1.5x oversampled grid (384^3), Kaiser-Bessel half width 2.5, density
compensation |k|^2: the large SENSE-CG configuration.  Seeded synthetic data:
200-ellipsoid phantom, Gaussian coil maps, k-space from this library's own
forward operator plus 0.5% complex Gaussian noise.

A step is one CG iteration (all 32 coils: E, E^H, FP64 dots and updates),
replayed from a captured CUDA graph with every input resident in HBM; each
iteration touches far more than L2 (the 384^3 x 32 grid alone is 14.5 GB), so
no flush is needed between steps.  `e2e` is the same metric through the C ABI
with host buffers: trajectory and k-space copied in, 30 CG iterations, image
copied back, all inside the timed region.

--impl reference times the CPU restatement of the reference algorithm (the
oracle; the reference itself cannot be built here) on the host cores: one
coil's E^H W E per step, scaled to a 32-coil iteration.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "SENSE-CG iter/s at 256³×32 coils, batched vs plain GPU, ≤1e-4 err vs FP64 oracle"
UNIT = "iter/s"
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="cg256")
    ap.add_argument("--e2e-solves", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain per-coil GPU path")
    ap.add_argument("--grid-mode", type=int, default=0,
                    help="gridding kernel (mrg_config.grid_mode): 0 fastest timed, 1 CUDA cores, 2 mma.sync, 3 tcgen05")
    ap.add_argument("--no-side-configs", dest="side_configs", action="store_false",
                    help="skip the throughput of the four smaller configurations")
    ap.add_argument("--profile-range", action="store_true",
                    help="bracket the two per-stage timing iterations with cudaProfilerStart/Stop "
                         "(for ncu --profile-from-start off: captures the launch shapes the bench runs)")
    ap.add_argument("--parity-full", action="store_true",
                    help="only the long parity runs against the CPU oracle (tens of minutes of CPU time): "
                         "SENSE-CG at 256^3 with 4 coils for 30 iterations and 32 coils for 3 iterations "
                         "against the FP64 oracle, FISTA at 128^3 x 16 coils for 100 iterations (fraction "
                         "and fixed threshold) against the FP32 oracle; prints one JSON object")
    ap.add_argument("--parity-legs", default="cg4,cg32,fista_fraction,fista_fixed",
                    help="comma-separated subset of the --parity-full legs")
    ap.add_argument("--kernel-case", default=None, choices=["wavelet_llr", "fft_tma"],
                    help="only a small case for one-kernel ncu captures: wavelet_llr runs three rounds of "
                         "mrg_wavelet (DB4, 3 levels) forward + inverse and the time low-rank threshold update "
                         "and pass (8^3 blocks) on a 10 x 128^3 stack through the C ABI; fft_tma runs three E "
                         "and E^H at 256 x 256 x 16 x 16 coils (384-point x and y lines) with the FFT passes "
                         "fixed to the persistent 16-thread kernels with tensor-map and bulk copies")
    ap.add_argument("--side-only", default=None, choices=["cg64", "fista128", "llr128", "grad96"],
                    help="run only this smaller configuration's throughput row (with --profile-range: its "
                         "timed iterations bracketed by cudaProfilerStart/Stop)")
    return ap.parse_args()


def workload(cfg_name):
    from mri_recon_gb300 import synth
    c = dict(synth.CONFIGS[cfg_name])
    N = c["N"]
    S = 16 * int(np.ceil(1.5 * N / 16))
    M = c["nproj"] * c["nread"]
    c.update(S=S, M=M)
    c["desc"] = ("SENSE-CG %d^3 x %d coils, 3D radial %d x %d (%.1fM samples/coil), %d^3 grid (1.5x), "
                 "Kaiser-Bessel half width 2.5, DCF |k|^2" % (N, c["coils"], c["nproj"], c["nread"], M / 1e6, S))
    return c


def bytes_model(c, nvalid):
    """Algorithmic HBM bytes per launch of each stage: every input read once and every output
    written once, a sample costing 16 B of trajectory (kx, ky, kz, kw) and 8 B per coil, a
    grid point 8 B per coil (the per-unit figures of the measurement plan).  Lists the
    implementation builds for itself (pair lists, tap tables) are not counted."""
    N, S, C = c["N"], c["S"], c["coils"]
    b = 8  # complex64
    img, smap = N ** 3 * b, N ** 3 * C * b
    t1, t2, g = N * N * S * C * b, N * S * S * C * b, S ** 3 * C * b
    y = nvalid * C * b
    return {
        "E_xfft_setimg": img + smap + t1,
        "E_zfft": t1 + t2,
        "E_yfft": t2 + g,
        "E_ungrid": g + nvalid * 16 + y,
        "EH_grid": y + nvalid * 16 + g,
        "EH_yfft": g + t2,
        "EH_zfft": t2 + t1,
        "EH_xfft_accum": t1 + smap + 2 * img,
    }


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of each stage's kernel
# in one ncu capture of the 256^3 x 32 workload's kernels at 1/8 of its size (128^3 x 32 coils,
# 16384 x 128 radial: `bench.py --config prof128 --profile-range` under
# `ncu --profile-from-start off --metrics dram__bytes_read.sum,dram__bytes_write.sum`), times 8,
# the growth of both the sample and the grid-point count.  Summary: profiles/ncu_traffic_cg256.md.
NCU_TRAFFIC_CG256 = {
    "E_xfft_setimg": 1.042e10, "E_zfft": 1.565e10, "E_yfft": 2.371e10, "E_ungrid": 2.385e10,
    "EH_grid": 3.875e10, "EH_yfft": 2.383e10, "EH_zfft": 1.577e10, "EH_xfft_accum": 1.099e10,
}


def bench_config(c, world):
    """The `config` object both arms print (identical keys and values for one workload)."""
    gb = c["S"] ** 3 * c["coils"] * 8 / 1e9
    return {"workload": c["desc"], "N": c["N"], "coils": c["coils"], "samples_per_coil": c["M"], "grid": c["S"],
            "iterations_per_solve": int(c.get("iters", 30)),
            "l2": "inputs larger than L2 (the %d^3 x %d grid is %.1f GB)" % (c["S"], c["coils"], gb),
            "parallelism": "replicas" if world > 1 else "single"}


STAGES = ["E_xfft_setimg", "E_zfft", "E_yfft", "E_ungrid", "EH_grid", "EH_yfft", "EH_zfft", "EH_xfft_accum"]


def kernel_of(stage, tuning, C):
    """Kernel that runs a stage, with the launch shape the autotuner picked."""
    if stage == "E_ungrid":
        if tuning["ungrid_lanes"] < 0:
            return "k_ungrid_mma<%d> (mma.sync TF32, 16 samples per warp, %d coils per pass)" % (
                -tuning["ungrid_lanes"], -4 * tuning["ungrid_lanes"])
        return "k_ungrid<%d,%d,%d>" % (tuning["ungrid_lanes"], max(tuning["ungrid_coils_per_lane"], 1),
                                      max(tuning.get("ungrid_rows_per_step", 1), 1))
    if stage == "EH_grid":
        cc = tuning["grid_coils_per_pass"]
        if cc <= -100:
            return "k_grid_umma<%d> (tcgen05 TF32, TMEM accumulators, %d coils per pass)" % (-cc - 100, -cc - 100)
        if cc < 0:
            return "k_grid_mma<%d> (mma.sync TF32, %d coils per pass)" % (-cc, -4 * cc)
        return "k_grid<%d> (FP32 CUDA cores)" % (cc if cc > 0 else min(C, 32))
    return {"E_xfft_setimg": "k_fft<Q,-1,SETIMG>", "E_yfft": "k_fft<Q,-1,PLAIN>", "E_zfft": "k_fft<Q,-1,PLAIN>",
            "EH_zfft": "k_fft<Q,+1,PLAIN>", "EH_yfft": "k_fft<Q,+1,PLAIN>",
            "EH_xfft_accum": "k_fft<Q,+1,ACCUM>"}[stage]


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            d = json.load(open(p))
            for k in ("hbm_gbs", "hbm_GBs", "hbm"):
                if k in d:
                    return float(d[k]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
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
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_sample(c, img, smap0, kx, ky, kz, kw, prec=0):
    """One coil's E^H W E at full size with the CPU restatement (OpenMP, all host threads);
    prec 0 is the FP32 restatement (the timed baseline), 1 its FP64 twin."""
    from oracle import oracle as O
    O.build()
    p = O.Plan(c["N"], prec=prec)
    frames = [dict(kx=kx, ky=ky, kz=kz, kw=kw, data=np.zeros((1, 1), np.complex64))]
    t0 = time.perf_counter()
    out = p.normal(frames, smap0[None], 0, img)
    dt = time.perf_counter() - t0
    return dt, out, O.num_threads()


def cpu_fft_split(c):
    """Seconds per coil of the FP32 restatement's two FFTs in one E^H W E (the pruned forward
    and the full inverse transform of the S^3 grid), and of the same two full transforms with
    scipy's pocketfft on all host threads, an FFTW-class library like the reference's."""
    import scipy.fft as sf
    from oracle import oracle as O
    O.build()
    p = O.Plan(c["N"], prec=0)
    L = O.lib()
    L.orc_fft3(p.h, -1)
    t0 = time.perf_counter()
    L.orc_fft3(p.h, -1)
    L.orc_fft3(p.h, +1)
    t_port = time.perf_counter() - t0
    del p
    g = np.zeros((c["S"],) * 3, np.complex64)
    workers = os.cpu_count() or 1
    g = sf.fftn(g, workers=workers, overwrite_x=True)
    t0 = time.perf_counter()
    g = sf.fftn(g, workers=workers, overwrite_x=True)
    g = sf.ifftn(g, workers=workers, overwrite_x=True)
    t_pocket = time.perf_counter() - t0
    return t_port, t_pocket


def cpu_vector_seconds(N):
    """Seconds of one CG iteration's vector updates (dots, X/R/P updates) at N^3 with the
    FP32 CPU restatement on all host threads."""
    from oracle import oracle as O
    O.build()
    rng = np.random.default_rng(5)
    shape = (N, N, N)
    R = [(rng.standard_normal(shape, np.float32) + 1j * rng.standard_normal(shape, np.float32)).astype(np.complex64)]
    P = [R[0].copy()]
    L = [(R[0] * np.complex64(0.5 + 0.25j)).astype(np.complex64)]
    X = [np.zeros(shape, np.complex64)]
    O.cg_vectors(X, R, P, L)
    t0 = time.perf_counter()
    O.cg_vectors(X, R, P, L)
    return time.perf_counter() - t0


def run_reference(a):
    """CPU arm: the oracle port of the reference algorithm on the host cores."""
    import torch.distributed as dist  # noqa: F401
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if rank != 0:
        return
    from mri_recon_gb300 import synth
    c = workload(a.config)
    N, C = c["N"], c["coils"]
    kx, ky, kz, kw = synth.radial_trajectory(N, c["nproj"], c["nread"])
    img = synth.phantom(N, c["ellipsoids"], seed=c["seed"])
    smap0 = synth.coil_map(N, C, 0, seed=c["seed"] + 1)
    vec_s = cpu_vector_seconds(N)
    times = []
    threads = 1
    for s in range(a.warmup + a.steps):
        dt, _, threads = cpu_sample(c, img, smap0, kx, ky, kz, kw)
        if s >= a.warmup:
            times.append(dt * C + vec_s)
    ms = 1000.0 * float(np.mean(times))
    value = 1000.0 / ms
    sample = ("per step: one coil's E^H W E (1 of %d coils) at %d^3 timed with the FP32 CPU restatement, x%d, plus "
              "one timed pass of the CG vector updates (%.3f s): one CG iteration" % (C, N, C, vec_s))
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": bench_config(c, world), "impl": "reference",
            "extrapolated_from": "1 of %d coils per step (the coils are independent and cost the same); ms_per_step "
                                 "is the projected time of one full iteration, not the time each step took" % C,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def caller_rows(p, img, c, dev, timed):
    """The callers either side of the operators on the 128^3 x 16-coil FISTA workload, each
    device-timed after one untimed call: low-resolution coil maps, Pipe density compensation
    of the trajectory, ESPIRiT maps and CLEAR iterations.  A failure is recorded, not raised."""
    import torch

    import mri_recon_gb300 as m
    from mri_recon_gb300 import synth
    out = {}
    N, C = c["N"], c["coils"]
    y = p.forward(0, img)
    kx, ky, kz, kw = synth.radial_trajectory(N, c["nproj"], c["nread"], seed=c["seed"])
    desc = "%d^3 x %d coils, %d x %d radial" % (N, C, c["nproj"], c["nread"])
    rows = [
        ("smaps_lowres128", "low-resolution coil maps (E^H per coil at k_rad 8, SOS normalisation), " + desc,
         "maps/s", 1, lambda: p.lowres_smaps(0, y, smap_res=8.0)),
        ("dcf128", "Pipe density compensation, 20 iterations, %d x %d radial at %d^3" % (c["nproj"], c["nread"], N),
         "runs/s", 1, lambda: m.dcf_pipe(kx, ky, kz, N)),
        ("espirit128", "ESPIRiT maps (kernel radius 3, calibration radius 12), " + desc, "maps/s", 1,
         lambda: p.espirit_smaps(0, y)),
    ]
    for name, metric, unit, n, fn in rows:
        try:
            fn()
            dt = timed(fn)
            out[name] = {"metric": metric, "value": n / dt, "unit": unit}
        except Exception as e:  # noqa: BLE001
            out[name] = {"metric": metric, "error": str(e)[:200]}
    try:
        X = torch.zeros((1, N, N, N), dtype=torch.complex64, device=dev)
        p.clear(m.clear_params(max_iter=1), X=X)
        t_lo = timed(lambda: p.clear(m.clear_params(max_iter=2), X=X))
        t_hi = timed(lambda: p.clear(m.clear_params(max_iter=6), X=X))
        out["clear128"] = {"metric": "CLEAR iter/s (per-coil gradient step, coil low rank on 4^3 blocks, "
                                     "4 block iterations), " + desc, "value": 4 / (t_hi - t_lo), "unit": "iter/s"}
    except Exception as e:  # noqa: BLE001
        out["clear128"] = {"metric": "CLEAR iter/s", "error": str(e)[:200]}
    return out


def iteration_bytes(N, C, Ms, fista=None):
    """Algorithmic HBM bytes of one iteration: per coil and frame of M samples one E^H W E
    costs 24 N^3 + 56 S^3 + 16 M bytes (maps read twice and the crop once, the oversampled
    grid written, transformed and read each way, samples written and read), plus per frame
    the trajectory read once per direction and 9 image passes of the vector updates.  FISTA
    adds per cycle spin a forward and an inverse wavelet (each level reads and writes its
    sub-box along x, y and z) and a soft threshold, and per iteration one magnitude pass and
    the bisection's counting passes (about 16) over 4-byte magnitudes.  fista: (spins,
    levels) or None."""
    S = 16 * int(np.ceil(1.5 * N / 16))
    n3 = N ** 3
    b = 0
    for M in Ms:
        b += C * (24 * n3 + 56 * S ** 3 + 16 * M) + 2 * 16 * M + 9 * 8 * n3
    if fista:
        spins, levels = fista
        T = len(Ms)
        wave = sum(3 * 2 * 8 * n3 / 8 ** l for l in range(levels))  # one direction, all levels
        b += T * (spins * (2 * wave + 2 * 8 * n3) + 8 * n3 + 16 * 4 * n3)
    return float(b)


def with_roofline(row, bytes_per, per_second):
    pk, kind = peaks()
    row["roofline"] = {"bound": "hbm", "algorithmic_bytes_per_unit": bytes_per,
                       "achieved_GBs": bytes_per * per_second / 1e9,
                       "frac": bytes_per * per_second / 1e9 / pk, "peak": pk, "peak_source": kind}
    return row


def side_configs(dev, only=None, profile=False):
    """Throughput of the four smaller configurations, device-timed with inputs resident:
    SENSE-CG 64^3 x 8 (iter/s), FISTA-wavelet 128^3 x 16 (iter/s), FISTA-wavelet + time
    low-rank 128^3 x 20 coils x 10 frames (iter/s), and the differentiable NUFFT at 96^3 x 8
    (loss + image and trajectory gradients per second, batch of 4 trajectories); plus the
    callers of the operators on the 128^3 x 16 workload (caller_rows)."""
    import torch

    import mri_recon_gb300 as m
    from mri_recon_gb300 import synth

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        if profile:
            torch.cuda.profiler.start()
        e0.record()
        fn()
        e1.record()
        torch.cuda.synchronize()
        if profile:
            torch.cuda.profiler.stop()
        return e0.elapsed_time(e1) / 1000.0

    def want(name):
        return only is None or only == name

    def setup(c, T, projs, jitter=0.0):
        N, C = c["N"], c["coils"]
        p = m.Plan(N, C, T)
        p.set_smaps(synth.coil_maps_torch(N, C, dev, seed=c["seed"] + 1))
        img = torch.from_numpy(synth.phantom(N, c["ellipsoids"], seed=c["seed"])).to(dev)
        start = 0
        for t in range(T):
            kx, ky, kz, kw = synth.radial_trajectory(N, int(projs[t]), c["nread"], start=start, jitter_grid=jitter,
                                                     seed=c["seed"] + t)
            start += int(projs[t])
            p.set_traj(t, kx, ky, kz, kw)
            y = p.forward(t, img)
            y += c["noise"] * float(y.abs().max()) * torch.complex(torch.randn_like(y.real), torch.randn_like(y.real))
            p.set_data(t, y)
        return p, img

    out = {}
    if want("cg64"):
        c = synth.CONFIGS["cg64"]
        p, _ = setup(c, 1, [c["nproj"]])
        X = torch.empty((1,) + p.ishape, dtype=torch.complex64, device=dev)
        p.cg_init(40, X)
        p.cg_iterate(3, X)
        dt = timed(lambda: p.cg_iterate(20, X))
        out["cg64"] = with_roofline({"metric": "SENSE-CG iter/s, 64^3 x 8 coils, 4096 x 64 radial", "value": 20 / dt,
                                     "unit": "iter/s"}, iteration_bytes(64, 8, [4096 * 64]), 20 / dt)
        del p

    def fista_rate(p, **kw):
        base = dict(max_eig_iter=30, cycle_spins=4, wave_levels=(3, 3, 3), wave_type=1, thresh=0.1, use_threshold=1)
        base.update(kw)
        if profile:  # the launches of a few iterations, bracketed for the profiler
            p.fista(m.fista_params(max_iter=2, **base))
            return 3 / timed(lambda: p.fista(m.fista_params(max_iter=3, **dict(base, max_eig_iter=0))))
        p.fista(m.fista_params(max_iter=2, **base))
        t_lo = timed(lambda: p.fista(m.fista_params(max_iter=5, **base)))
        t_hi = timed(lambda: p.fista(m.fista_params(max_iter=25, **base)))
        return 20 / (t_hi - t_lo)

    if want("fista128"):
        c = synth.CONFIGS["fista128"]
        p, img = setup(c, 1, [c["nproj"]])
        rate = fista_rate(p)
        out["fista128"] = with_roofline({"metric": "FISTA-wavelet iter/s, 128^3 x 16 coils, 16384 x 128 radial, db4 3 "
                                                   "levels, 4 cycle spins, fraction threshold 0.1", "value": rate,
                                         "unit": "iter/s"},
                                        iteration_bytes(128, 16, [16384 * 128], fista=(4, 3)), rate)
        if only is None:
            out.update(caller_rows(p, img, c, dev, timed))
        del p
    if want("llr128"):
        c = synth.CONFIGS["llr128"]
        projs = synth.frame_projection_counts(c["frames"], c["proj_lo"], c["proj_hi"], c["seed"])
        p, _ = setup(c, c["frames"], projs)
        rate = fista_rate(p, llr_block=(8, 8, 8), llr_block_iter=4, llr_alpha=0.001)
        # the low-rank step adds one read and write of the 10 frames per block pass (5 passes)
        llr_b = iteration_bytes(128, 20, [int(n) * 128 for n in projs], fista=(4, 3)) + 5 * 2 * 8 * 128 ** 3 * 10
        out["llr128"] = with_roofline({"metric": "FISTA-wavelet + time low-rank iter/s, 128^3 x 20 coils x 10 "
                                                 "frames (1500-3500 projections each), 8^3 blocks", "unit": "iter/s",
                                       "value": rate}, llr_b, rate)
        del p
    if want("grad96"):
        c = synth.CONFIGS["grad96"]
        p, img = setup(c, c["batch"], [c["nproj"]] * c["batch"], jitter=c["jitter"])
        ys = [torch.randn((c["coils"], p.M[t]), dtype=torch.complex64, device=dev) for t in range(c["batch"])]

        def grads():
            for t in range(c["batch"]):
                p.grad(t, img, ys[t])
        grads()
        dt = timed(lambda: [grads() for _ in range(3)])
        # one evaluation: E and E^H of one 96^3 x 8-coil frame (the operator bytes of one iteration
        # without the CG vector passes) plus the gradient's extra trajectory and sample traffic
        gb = iteration_bytes(96, 8, [6000 * 96]) - 9 * 8 * 96 ** 3 + 8 * 16 * 6000 * 96
        out["grad96"] = with_roofline({"metric": "differentiable NUFFT evaluations/s (loss, image and trajectory "
                                                 "gradients), 96^3 x 8 coils, 6000 x 96 jittered radial",
                                       "value": 3 * c["batch"] / dt, "unit": "evals/s"}, gb, 3 * c["batch"] / dt)
        del p
    torch.cuda.synchronize()
    return out


def rel_l2(a, b):
    a = np.asarray(a).astype(np.complex128)
    b = np.asarray(b).astype(np.complex128)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def parity_cg64(dev):
    """SENSE-CG at 64^3 x 8 coils, 4096 x 64 radial, 20 iterations, k-space from an FP64
    direct NUDFT of the 10-ellipsoid phantom times each coil map plus 1% noise: the GPU
    (batched, graph-replayed) against the FP64 and FP32 CPU oracle."""
    import torch

    import mri_recon_gb300 as m
    from mri_recon_gb300 import synth
    from oracle import oracle as O
    O.build()
    c = synth.CONFIGS["cg64"]
    N, C, iters = c["N"], c["coils"], c["iters"]
    kx, ky, kz, kw = synth.radial_trajectory(N, c["nproj"], c["nread"], seed=c["seed"])
    img = synth.phantom(N, c["ellipsoids"], seed=c["seed"])
    smaps = synth.coil_maps(N, C, seed=c["seed"] + 1)
    y = synth.add_noise(synth.nudft_torch(img[None] * smaps, kx, ky, kz, dev).astype(np.complex64), c["noise"],
                        c["seed"] + 2)
    p = m.Plan(N, C, 1)
    p.set_traj(0, kx, ky, kz, kw)
    p.set_smaps(torch.from_numpy(smaps).to(dev))
    p.set_data(0, torch.from_numpy(y).to(dev))
    X, _ = p.cg(iters)
    X = X[0].cpu().numpy()
    fr = [dict(kx=kx, ky=ky, kz=kz, kw=kw, data=y)]
    X64, _ = O.Plan(N, prec=1).cg(fr, smaps, iters)
    X32, _ = O.Plan(N, prec=0).cg(fr, smaps, iters)
    return {"scope": "SENSE-CG 64^3 x 8 coils, 4096 x 64 radial, %d iterations, data from an FP64 direct NUDFT" % iters,
            "rel_l2_vs_fp64_oracle": rel_l2(X, X64[0]), "rel_l2_vs_fp32_oracle": rel_l2(X, X32[0]),
            "fp32_oracle_vs_fp64_oracle": rel_l2(X32[0], X64[0]), "bound": 1e-4}


def parity_full(dev, legs):
    """The long parity runs (CPU oracle on the host cores; tens of minutes).  legs: the
    subset of cg4, cg32, fista_fraction, fista_fixed to run."""
    import torch

    import mri_recon_gb300 as m
    from mri_recon_gb300 import synth
    from oracle import oracle as O
    O.build()
    out = {}
    t0 = time.perf_counter()
    c = workload("cg256")
    N, C = c["N"], c["coils"]
    kx, ky, kz, kw = synth.radial_trajectory(N, c["nproj"], c["nread"])
    img = synth.phantom(N, c["ellipsoids"], seed=c["seed"])
    smaps = synth.coil_maps_torch(N, C, dev, seed=c["seed"] + 1).cpu().numpy()
    fr = dict(kx=kx, ky=ky, kz=kz, kw=kw)

    def gpu_cg(maps, y, iters):
        p = m.Plan(N, len(maps), 1)
        p.set_traj(0, kx, ky, kz, kw)
        p.set_smaps(torch.from_numpy(np.ascontiguousarray(maps)).to(dev))
        p.set_data(0, torch.from_numpy(y).to(dev))
        X, r = p.cg(iters)
        X = X[0].cpu().numpy()
        del p
        torch.cuda.empty_cache()
        return X, r

    # (A) 4 of the 32 coils, 30 iterations; k-space from the FP64 oracle with a wide kernel
    # (half width 6 on a 2x grid), not from the operator under test, plus 0.5% noise
    if "cg4" in legs:
        out.update(parity_cg4(O, gpu_cg, N, c, kx, ky, kz, kw, img, smaps, fr, t0))
    if "cg32" in legs:
        out.update(parity_cg32(O, gpu_cg, N, C, c, kx, ky, kz, kw, img, smaps, fr))
    del smaps
    for leg, use_threshold, thresh in (("fista_fraction", 1, 0.1), ("fista_fixed", 2, 0.006)):
        if leg in legs:
            out.update(parity_fista128(O, m, dev, use_threshold, thresh))
    return out


def parity_cg4(O, gpu_cg, N, c, kx, ky, kz, kw, img, smaps, fr, t0):
    from mri_recon_gb300 import synth
    out = {}
    wide = O.Plan(N, overgrid=2.0, dwin=6.0, prec=1)
    y4 = np.stack([wide.forward(img, smaps[k], kx, ky, kz, kw) for k in range(4)]).astype(np.complex64)
    del wide
    y4 = synth.add_noise(y4, c["noise"], c["seed"] + 2)
    X, r = gpu_cg(smaps[:4], y4, 30)
    X64, r64 = O.Plan(N, prec=1).cg([dict(fr, data=y4)], smaps[:4], 30)
    out["cg256_4coils_30it"] = {
        "scope": "SENSE-CG 256^3, coils 0-3 of the 32 maps, 65536 x 256 radial, 30 iterations; data: FP64 "
                 "wide-kernel (half width 6, 2x grid) oracle E plus 0.5% noise",
        "rel_l2_vs_fp64_oracle": rel_l2(X, X64[0]), "residual_rel_diff_last": float(abs(r[-1] - r64[-1]) / r64[-1]),
        "bound": 1e-4, "seconds": time.perf_counter() - t0}
    print(json.dumps(out), flush=True)
    return out


def parity_cg32(O, gpu_cg, N, C, c, kx, ky, kz, kw, img, smaps, fr):
    # (B) all 32 coils, 3 iterations; data from the FP64 oracle E
    from mri_recon_gb300 import synth
    out = {}
    t1 = time.perf_counter()
    o64 = O.Plan(N, prec=1)
    y = np.stack([o64.forward(img, smaps[k], kx, ky, kz, kw) for k in range(C)]).astype(np.complex64)
    y = synth.add_noise(y, c["noise"], c["seed"] + 3)
    X, r = gpu_cg(smaps, y, 3)
    X64, r64 = o64.cg([dict(fr, data=y)], smaps, 3)
    del o64
    out["cg256_32coils_3it"] = {
        "scope": "SENSE-CG 256^3 x 32 coils, 65536 x 256 radial, 3 iterations; data: FP64 oracle E plus 0.5% noise",
        "rel_l2_vs_fp64_oracle": rel_l2(X, X64[0]), "bound": 1e-4, "seconds": time.perf_counter() - t1}
    print(json.dumps(out), flush=True)
    return out


def parity_fista128(O, m, dev, use_threshold, thresh):
    """(C) FISTA 128^3 x 16 coils, 100 iterations, against the FP32 oracle: the fraction
    threshold 0.1 of the configuration (a bisection end point, discontinuous in its input) and
    a fixed threshold (continuous)."""
    import torch
    from mri_recon_gb300 import synth
    t2 = time.perf_counter()
    c2 = synth.CONFIGS["fista128"]
    N2, C2 = c2["N"], c2["coils"]
    kx, ky, kz, kw = synth.radial_trajectory(N2, c2["nproj"], c2["nread"], seed=c2["seed"])
    img = synth.phantom(N2, c2["ellipsoids"], seed=c2["seed"])
    maps = synth.coil_maps(N2, C2, seed=c2["seed"] + 1)
    o64 = O.Plan(N2, prec=1)
    y = np.stack([o64.forward(img, maps[k], kx, ky, kz, kw) for k in range(C2)]).astype(np.complex64)
    y = synth.add_noise(y, c2["noise"], c2["seed"] + 2)
    p = m.Plan(N2, C2, 1)
    p.set_traj(0, kx, ky, kz, kw)
    p.set_smaps(torch.from_numpy(maps).to(dev))
    p.set_data(0, torch.from_numpy(y).to(dev))
    kwp = dict(max_iter=100, max_eig_iter=30, cycle_spins=4, wave_levels=(3, 3, 3), wave_type=1, thresh=thresh,
               use_threshold=use_threshold)
    X, _, step = p.fista(m.fista_params(**kwp))
    X = X[0].cpu().numpy()
    q = O.FistaParams()
    q.max_iter, q.max_eig_iter, q.cycle_spins = 100, 30, 4
    q.wave_levels[:] = [3, 3, 3]
    q.wave_type, q.thresh, q.use_threshold = 1, thresh, use_threshold
    q.llr_bs[:] = [4, 4, 4]
    q.llr_block_iter, q.llr_alpha, q.clear_amp, q.clear_t2 = 4, 0.0, 4.0, 6.0
    q.rand_skip = 2 * N2 ** 3
    X32, _, s32, _ = O.Plan(N2, prec=0).fista([dict(kx=kx, ky=ky, kz=kz, kw=kw, data=y)], maps, q)
    name = "fraction 0.1" if use_threshold == 1 else "fixed threshold %g" % thresh
    out = {}
    out["fista128_16coils_100it_" + ("fraction" if use_threshold == 1 else "fixed")] = {
        "scope": "FISTA-wavelet 128^3 x 16 coils, 16384 x 128 radial, db4 3 levels, 4 cycle spins, %s, "
                 "100 iterations; data: FP64 oracle E plus 1%% noise" % name,
        "rel_l2_vs_fp32_oracle": rel_l2(X, X32[0]), "step_rel_diff": abs(step - s32) / s32,
        # the fraction threshold jumps where a coefficient count crosses a bisection branch, so
        # 1e-7 input perturbations move the FP32 oracle itself by up to 2.5e-4 after 100
        # iterations; the fixed threshold is continuous and held to the stated 1e-4
        "bound": 1e-4 if use_threshold == 2 else 2e-3,
        "seconds": time.perf_counter() - t2}
    return out


def kernel_case_wavelet_llr():
    """10 frames of 128^3 (168 MB): the regulariser kernels of the gated FISTA configuration."""
    import ctypes

    import torch

    import mri_recon_gb300 as m
    L = m.load()
    ip = lambda v: (ctypes.c_int * 3)(*v)  # noqa: E731
    g = torch.Generator(device="cuda").manual_seed(1)
    X = torch.randn((10, 128, 128, 128), dtype=torch.complex64, device="cuda", generator=g)
    p = ctypes.c_void_p(X.data_ptr())
    smax = ctypes.c_float()
    for rep in range(3):
        for inv in (0, 1):
            if L.mrg_wavelet(p, 10, 128, 128, 128, ip((3, 3, 3)), ip((1, 2, 3)), 1, inv, None) != 0:
                raise RuntimeError(L.mrg_last_error().decode())
        if L.mrg_llr_update_threshold(p, 10, 128, 128, 128, ip((8, 8, 8)), 4.0, 6.0, 2, ctypes.byref(smax), None) != 0:
            raise RuntimeError(L.mrg_last_error().decode())
        if L.mrg_llr_thresh(p, 10, 128, 128, 128, ip((8, 8, 8)), 4, 0.0, smax, 1000 * rep, None) != 0:
            raise RuntimeError(L.mrg_last_error().decode())
    torch.cuda.synchronize()
    print(json.dumps({"kernel_case": "wavelet_llr", "smax": smax.value}), flush=True)


def kernel_case_fft_tma():
    """E and E^H on a 384 x 384 x 32 grid of 16 coils (0.6 GB): the x passes (set_image,
    accumulate) and y passes run the persistent kernels with 16 threads per line and their
    tiles copied by tensor maps / bulk copies (FFT tuning fixed to xp = 2 | 4, 16 lines per CTA)."""
    import torch

    import mri_recon_gb300 as m
    from mri_recon_gb300 import synth
    N, C = (256, 256, 16), 16
    rng = np.random.default_rng(5)
    M = 400000
    kx, ky, kz = [rng.uniform(-n / 2, n / 2, M).astype(np.float32) for n in N]
    kw = (kx.astype(np.float64) ** 2 + ky ** 2 + kz ** 2).astype(np.float32)
    p = m.Plan(N, C, 1)
    p.set_fft_tuning(ib=[16] * 6, xp=[6] * 6)  # before the first trajectory: no FFT tuning
    p.set_traj(0, kx, ky, kz, kw)
    ishape = (N[2], N[1], N[0])
    g = torch.Generator(device="cuda").manual_seed(2)
    maps = torch.randn((C,) + ishape, dtype=torch.complex64, device="cuda", generator=g)
    p.set_smaps(maps)
    X = torch.randn(ishape, dtype=torch.complex64, device="cuda", generator=g)
    for _ in range(3):
        y = p.forward(0, X)
        Xh = p.adjoint(0, y, torch.zeros(ishape, dtype=torch.complex64, device="cuda"))
    torch.cuda.synchronize()
    print(json.dumps({"kernel_case": "fft_tma", "fft_tuning": p.fft_tuning(), "norm": float(Xh.abs().sum())}),
          flush=True)


def run_ours(a):
    import torch
    import torch.distributed as dist

    if a.kernel_case:
        torch.cuda.set_device(0)
        {"wavelet_llr": kernel_case_wavelet_llr, "fft_tma": kernel_case_fft_tma}[a.kernel_case]()
        return

    if a.parity_full:
        torch.cuda.set_device(0)
        legs = [x for x in a.parity_legs.split(",") if x]
        print(json.dumps(parity_full(torch.device("cuda", 0), legs)), flush=True)
        return

    if a.side_only:
        torch.cuda.set_device(0)
        print(json.dumps(side_configs(torch.device("cuda", 0), only=a.side_only, profile=a.profile_range)),
              flush=True)
        return

    import mri_recon_gb300 as m
    from mri_recon_gb300 import replicas, synth

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    st = torch.cuda.current_stream()
    L = m.load()

    c = workload(a.config)
    N, C, M = c["N"], c["coils"], c["M"]
    kx, ky, kz, kw = synth.radial_trajectory(N, c["nproj"], c["nread"])
    img = synth.phantom(N, c["ellipsoids"], seed=c["seed"])
    smaps = synth.coil_maps_torch(N, C, dev, seed=c["seed"] + 1)
    plan = m.Plan(N, C, 1, grid_mode=a.grid_mode)
    plan.set_traj(0, kx, ky, kz, kw)
    plan.set_smaps(smaps)
    x_true = torch.from_numpy(img).to(dev)
    y = plan.forward(0, x_true)                                    # (C, M) on the device
    gen = torch.Generator(device=dev).manual_seed(c["seed"])
    sig = c["noise"] * float(y.abs().max())
    y += sig * torch.complex(torch.randn(y.shape, generator=gen, device=dev),
                             torch.randn(y.shape, generator=gen, device=dev))
    plan.set_data(0, y)
    torch.cuda.synchronize()

    # --- device-resident timed region: K CG iterations replayed from a graph ---
    X = torch.empty((1, N, N, N), dtype=torch.complex64, device=dev)
    plan.cg_init(a.warmup + a.steps + 8, X)
    plan.cg_iterate(a.warmup, X)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = Clocks(local)
    clk.start()
    l0 = L.mrg_kernel_launches()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    plan.cg_iterate(a.steps, X)
    e1.record(st)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ms_local = e0.elapsed_time(e1)
    launches = L.mrg_kernel_launches() - l0
    clocks = clk.stop()
    value, s_max = replicas.job_throughput(a.steps, ms_local / 1000.0, dev)
    ms = 1000.0 * s_max / a.steps
    resid = plan.cg_residuals(a.warmup + a.steps)

    # --- per-stage timing (eager, events between stages) for the roofline ---
    plan.set_timing(True)
    if a.profile_range:
        torch.cuda.profiler.start()
    plan.cg_iterate(2, X, use_graph=False)
    torch.cuda.synchronize()
    if a.profile_range:
        torch.cuda.profiler.stop()
    tms, calls = plan.timings()
    plan.set_timing(False)
    fi = plan.frame_info(0, taps=True)
    bm = bytes_model(c, fi["nvalid"])
    out_tuning = plan.frame_tuning(0)
    per_launch_ms = {s: float(tms[i]) / max(calls, 1) for i, s in enumerate(STAGES)}
    dom = max(per_launch_ms, key=per_launch_ms.get)
    peak, peak_kind = peaks()
    achieved = bm[dom] / (per_launch_ms[dom] / 1000.0) / 1e9
    # the measurement plan's B_iter (one read and one write per 3D FFT); the per-stage sum of the
    # pruned three-pass FFTs is reported beside it
    iter_bytes = iteration_bytes(N, C, [c["M"]])
    stage_bytes = sum(bm.values()) + 9 * N ** 3 * 8
    roofline = {"bound": "hbm", "kernel": kernel_of(dom, out_tuning, C), "stage": dom, "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": NCU_TRAFFIC_CG256.get(dom) if a.config == "cg256" else None,
                "algorithmic_bytes_per_launch": bm[dom],
                "launch_ms": per_launch_ms[dom]}
    # The ungridding gather is bound by the L1 data path, not HBM: every sample reads its
    # nx*ny*nz taps x C coils (8 B each) through L1.  Nominal L1 load bandwidth: 128 B per
    # clock per SM, at the SM clock sampled during the timed region.
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    l1_peak = 152 * 128 * sm_mhz * 1e6 / 1e9
    gather = fi["ntaps"] * C * 8
    if out_tuning["ungrid_lanes"] > 0:  # the CUDA-core kernel (the tensor-core one loads each value once per 16 samples)
        roofline["ungrid_l1_gather"] = {"bytes_per_launch": gather, "achieved": gather / (per_launch_ms["E_ungrid"] / 1e3) / 1e9,
                                        "peak": l1_peak, "unit": "GB/s",
                                        "frac": gather / (per_launch_ms["E_ungrid"] / 1e3) / 1e9 / l1_peak,
                                        "peak_source": "nominal 128 B/clk/SM x 152 SMs at the sampled SM clock",
                                        "taps_per_sample": fi["ntaps"] / max(fi["nvalid"], 1)}
    iteration_roofline = {"bytes_per_iter": iter_bytes, "achieved_GBs": iter_bytes * value / world / 1e9,
                          "frac": iter_bytes * value / world / 1e9 / peak, "peak_source": peak_kind,
                          "bytes_per_iter_stages": stage_bytes, "stage_ms": per_launch_ms}

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
           "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic",
           "config": bench_config(c, world), "graph": "one CG iteration per CUDA graph replay",
           "gpu_launches": int(launches), "roofline": roofline, "iteration_roofline": iteration_roofline,
           "autotune": out_tuning, "fft_tuning": plan.fft_tuning(),
           "cg_residual_first_last": [float(resid[0]), float(resid[-1])]}
    if clocks:
        out["clocks"] = clocks

    # --- plain per-coil GPU path: one coil per call, as the reference's coil loop ---
    if not a.no_plain and rank == 0:
        pp = m.Plan(N, 1, 1)
        pp.set_traj(0, *[torch.from_numpy(v).to(dev) for v in (kx, ky, kz, kw)])
        ytmp = torch.empty(M, dtype=torch.complex64, device=dev)
        Lh = torch.zeros((N, N, N), dtype=torch.complex64, device=dev)
        P0 = X[0]
        pp.forward_coil(0, P0, smaps[0], ytmp)
        pp.adjoint_coil(0, smaps[0], ytmp, Lh)
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record(st)
        for cc in range(C):
            pp.forward_coil(0, P0, smaps[cc], ytmp)
            pp.adjoint_coil(0, smaps[cc], ytmp, Lh)
        p1.record(st)
        torch.cuda.synchronize()
        plain_ms = p0.elapsed_time(p1)
        out["plain_gpu"] = {"value": 1000.0 / plain_ms, "unit": UNIT, "ms_per_iter": plain_ms,
                            "note": "per-coil E then E^H through the C ABI (operators only; CG vector updates "
                                    "excluded), same kernels with one coil per call",
                            "batched_over_plain": value / world / (1000.0 / plain_ms)}
        # parity of the per-coil operator at full size against the FP32 CPU restatement (coil 0)
        if not a.no_cpu:
            Lh.zero_()
            xin = torch.from_numpy(img).to(dev)
            pp.forward_coil(0, xin, smaps[0], ytmp)
            pp.adjoint_coil(0, smaps[0], ytmp, Lh)
            gpu0 = Lh.cpu().numpy()
            smap0 = smaps[0].cpu().numpy()
            dt, ref0, threads = cpu_sample(c, img, smap0, kx, ky, kz, kw)
            vec_s = cpu_vector_seconds(N)
            cpu_val = 1.0 / (dt * C + vec_s)
            out["cpu_baseline"] = {"value": cpu_val, "unit": UNIT, "cores": threads, "kind": "port",
                                   "sample": "one coil's E^H W E (1 of %d) at %d^3 with the FP32 CPU restatement "
                                             "(OpenMP), x%d, plus the CG vector updates (%.3f s) = one CG iteration"
                                             % (C, N, C, vec_s)}
            try:  # how much of the port's time its own FFT takes, against an FFTW-class FFT
                t_port, t_pocket = cpu_fft_split(c)
                out["cpu_baseline"]["fft_s_per_coil"] = t_port
                out["cpu_baseline"]["pocketfft_s_per_coil"] = t_pocket
                out["cpu_baseline"]["value_with_pocketfft"] = 1.0 / ((max(dt - t_port, 0.0) + t_pocket) * C + vec_s)
            except Exception as e:  # noqa: BLE001
                out["cpu_baseline"]["fft_split_error"] = str(e)[:200]
            _, ref64, _ = cpu_sample(c, img, smap0, kx, ky, kz, kw, prec=1)

            def rl(a, b):
                return float(np.linalg.norm(a - b) / np.linalg.norm(b))
            out["parity"] = {"cg256_operator": {
                "rel_l2_vs_fp32_oracle": rl(gpu0, ref0), "rel_l2_vs_fp64_oracle": rl(gpu0, ref64),
                "fp32_oracle_vs_fp64_oracle": rl(ref0, ref64), "bound": 1e-5,
                "scope": "E^H W E, coil 0, %d^3, full trajectory" % N}}
            try:
                out["parity"]["cg64_20it"] = parity_cg64(dev)
            except Exception as e:  # noqa: BLE001
                out["parity"]["cg64_20it"] = {"error": str(e)[:200]}
        del pp

    # --- e2e through the C ABI with host buffers ---
    if a.e2e_solves > 0:
        iters = int(c.get("iters", 30))
        y_host = y.cpu().pin_memory()
        traj_host = [torch.from_numpy(v).pin_memory() for v in (kx, ky, kz, kw)]
        X_host = torch.empty((1, N, N, N), dtype=torch.complex64).pin_memory()
        del y
        times, phases = [], []
        for s in range(1 + a.e2e_solves):
            torch.cuda.synchronize()
            if world > 1:
                dist.barrier()
            t0 = time.perf_counter()
            plan.set_traj(0, *traj_host)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            plan.set_data(0, y_host)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            plan.cg(iters, X=X_host, use_graph=True)
            torch.cuda.synchronize()
            if s > 0:
                t3 = time.perf_counter()
                times.append(t3 - t0)
                phases.append({"set_traj_s": t1 - t0, "set_data_s": t2 - t1, "cg_s": t3 - t2})
        e2e_val, _ = replicas.job_throughput(iters, max(times), dev)
        out["e2e"] = {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": int(C * M * 8 + 4 * M * 4),
                      "d2h_bytes_per_step": int(N ** 3 * 8 + iters * 8),
                      "step": "one %d-iteration solve: trajectory + k-space host->device, set-up, CG, image "
                              "device->host" % iters, "phases": phases[-1] if phases else None}
    if a.side_configs and rank == 0:
        del plan
        torch.cuda.empty_cache()
        out["other_configs"] = side_configs(dev)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out), flush=True)


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
