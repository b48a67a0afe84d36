"""Benchmark of the photon-propagation path on one GB300 (or N replicas).

Workload (the plain-octree AMR configuration): a 256^3 periodic base field
(octree level 10, file level 8) refined to octree level 14 inside 2000 seeded
NFW haloes; 1000 x 1000 rays on a regular grid filling a 10 x 10 degree cone,
integrated to z = 2 with TSC interpolation, 8 steps per cell and the
infinitesimal lensing Jacobian at z = 2.  Inputs are seeded synthetic data
with those shapes (no simulation data are available).

One step = one batch of rays (whole 8 x 4 sky tiles drawn at random from the
grid, so every batch samples the whole cone).  The octree (GBs) is larger
than L2, so no flush is needed between steps.

Metric: RK4 photon-steps per second (one accepted RK4 step of one ray =
one photon-step, src/integrator.h:776).

--mode surrogate measures the learned field surrogate (a third line): the
64^3 field at octree level 8 over a 5 x 5 degree cone to z = 2, 1000 x 1000
rays, the network trained on 50M octree-labelled samples first; value = the
surrogate form's photon-steps/s with flagged rays re-run on the octree, with
the plain octree path on the same rays and the measured deflection error
beside it.

--mode catalogue measures the catalogue root-finder instead (a second JSON
line, not the headline): one step = one batch of sources on the same octree,
uniform in comoving volume inside the cone out to z = 2, solved to
cat_accuracy = 1e-8 (Catalogues::iterateNewtonMethod, at most 11 rays per
source); metric sources/s, with the photon-steps/s over all rounds beside it.
"""
from __future__ import annotations

import argparse
import ctypes as C
import hashlib
import importlib
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)
PKG = "magrathea-pathfinder_gb300"

METRIC = "RK4 photon-steps/s on 1 GB300, surrogate vs plain octree, at <=1e-3 rel deflection"
UNIT = "photon-steps/s"
# payload bytes requested per photon-step, TSC + Jacobian: 4 RK stages x 27 cells x 16 B
# + post-step 27 x 28 B + Jacobian 6 x 27 x 12 B
BYTES_PER_PHOTON_STEP = 4 * 27 * 16 + 27 * 28 + 6 * 27 * 12
# DRAM bytes per photon-step of the propagate kernel, from one ncu capture of the
# same kernel on the medium octree (65 536 rays to z = 0.5): (37.66 + 1.93) MB
# over 6.95e7 photon-steps; the bench's per-launch traffic is this figure times
# the photon-steps of a launch
DRAM_BYTES_PER_PHOTON_STEP = 0.57
# FP64 add + fma + mul thread operations per photon-step of the same capture
# (smsp__sass_thread_inst_executed_op_{dadd,dfma,dmul}_pred_on): the
# arithmetic that bounds the kernel on this part, whose FP64 pipe retires 2
# operations per SM per cycle (sm__sass_thread_inst_executed_op_dfma_pred_on
# .sum.peak_sustained = 304 per cycle for 152 SMs)
FP64_OPS_PER_PHOTON_STEP = 137
FP64_OPS_PER_SM_CYCLE = 2


def fp64_roofline(photon_steps_per_s, clocks):
    """FP64 arithmetic throughput of the propagate kernel against the part's
    FP64 peak at the SM clock sampled during the timed region."""
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    sms = 152
    try:
        import torch
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    except Exception:
        pass
    peak = sms * FP64_OPS_PER_SM_CYCLE * mhz * 1e6 / 1e12
    achieved = photon_steps_per_s * FP64_OPS_PER_PHOTON_STEP / 1e12
    return {"achieved": achieved, "peak": peak, "unit": "TFLOP/s (FP64 add/fma/mul thread ops)", "frac": achieved / peak,
            "ops_per_photon_step": FP64_OPS_PER_PHOTON_STEP,
            "source": "ops per photon-step from the ncu capture of the medium octree; peak = SMs x 2 x sampled SM clock"}


def workload_spec(synth, workload: str):
    cosmo = synth.Cosmology()
    chi2 = float(cosmo.chi_of_z(2.0)[0])
    if workload == "small":
        return synth.OctreeSpec(base_level=8, box_cells=64, lbox=2048.0, half_y=5.0, half_z=5.0, chi_max=chi2 * 1.02,
                                halos=50, max_level=11, refine_cells=2.5, seed=42)
    if workload == "medium":   # the same construction one level coarser: larger than L2, ~1 GB on the device
        return synth.OctreeSpec(base_level=9, box_cells=128, lbox=2048.0, half_y=5.0, half_z=5.0, chi_max=chi2 * 1.02,
                                halos=500, max_level=13, mass_min=1e12, mass_max=1e15, refine_cells=4.5, seed=42)
    return synth.OctreeSpec(base_level=10, box_cells=256, lbox=2048.0, half_y=5.0, half_z=5.0, chi_max=chi2 * 1.02,
                            halos=2000, max_level=14, mass_min=1e12, mass_max=1e15, refine_cells=4.5, seed=42)


def octree_records(synth, spec):
    key = hashlib.sha1(repr(spec).encode()).hexdigest()[:16]
    path = os.path.join(os.environ.get("TMPDIR", "/tmp"), "mpf_bench_%s.bin" % key)
    if os.path.exists(path):
        return synth.read_bin(path)
    rec = synth.make_octree(spec)
    tmp = path + ".%d" % os.getpid()
    synth.write_bin(tmp, rec)
    os.replace(tmp, path)
    return rec


def ray_grid(n_side=1000, half_deg=5.0, tile=(8, 4), seed=0):
    """Launch records of the n_side^2 grid, reordered by shuffled 8x4 tiles."""
    t = (np.arange(n_side) + 0.5) / n_side * 2.0 - 1.0
    ph = np.radians(half_deg) * t
    th = np.pi / 2 + np.radians(half_deg) * t
    ty, tz = tile
    ny, nz = n_side // ty, n_side // tz
    rng = np.random.default_rng(seed)
    order = rng.permutation(ny * nz)
    iy = (order // nz)[:, None] * ty + (np.arange(ty * tz) % ty)[None, :]
    iz = (order % nz)[:, None] * tz + (np.arange(ty * tz) // ty)[None, :]
    P, T = ph[iy.ravel()], th[iz.ravel()]
    out = np.zeros((P.shape[0], 6))
    out[:, 3] = np.sin(T) * np.cos(P)
    out[:, 4] = np.sin(T) * np.sin(P)
    out[:, 5] = np.cos(T)
    return out


def cosmology_table(synth):
    return synth.Cosmology().conformal_table(n=4000, amin=0.05)


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join(os.environ.get("TMPDIR", "/tmp"), "mpf_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_baseline(oracle_mod, records, cos, length, launch, planes, per_thread=24, seed=1):
    """The C oracle (restated reference algorithm, binary search over sorted
    keys, trajectory then Jacobian post-pass) on a bounded random sample.
    Returns the baseline entry and the sample with the oracle's outputs
    (launch records, steps, final records, surface records)."""
    nthreads = os.cpu_count() or 1
    O = oracle_mod.Oracle(records, {"t": cos[0], "a": cos[1], "dadt": cos[2]}, length, nthreads=nthreads)
    rng = np.random.default_rng(seed)
    idx = rng.choice(launch.shape[0], size=per_thread * nthreads, replace=False)
    sample = np.ascontiguousarray(launch[idx])
    t0 = time.perf_counter()
    steps, final, pl = O.propagate(sample, order=2, nsteps=8, stop="redshift", planes=planes, jacobian=True)
    dt = time.perf_counter() - t0
    total = int(steps.sum())
    entry = {"value": total / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
             "sample": "%d rays drawn from the grid, %d photon-steps, %.1f s, %d threads (C oracle, Jacobian post-pass)"
                       % (idx.shape[0], total, dt, nthreads)}
    return entry, (sample, steps, final, pl)


def parity_entry(pkg, tree, cosmo, length, planes, oracle_run, exact=False):
    """The benchmarked kernel on the oracle's sample rays, compared output by
    output with the oracle (the reference's float64 algorithm)."""
    acc = importlib.import_module(PKG + ".accuracy")
    sample, s_ref, f_ref, p_ref = oracle_run
    s, f, pl, _ = pkg.propagate(tree, cosmo, sample, length, nsteps=8, order=2, stop="redshift", planes=planes,
                                jacobian=True, exact=exact)
    rep = acc.compare(sample, s, f, pl, s_ref, f_ref, p_ref)
    rep["against"] = "C oracle (the reference's float64 algorithm, bit-exact with its own build on the fixtures)"
    rep["tolerance"] = {"deflection_rel": 1e-6, "redshift_rel": 1e-6, "lensing_of_scale": 1e-6}
    rep["within_tolerance"] = bool(acc.within(rep))
    return rep


CAT_METRIC = "catalogue sources/s (Newton root-finder to cat_accuracy 1e-8, TSC, <=11 rays per source)"
CAT_UNIT = "sources/s"
# payload bytes per photon-step without the lensing Jacobian (rounds 0-1 of the root-finder)
BYTES_PER_PHOTON_STEP_NOJAC = 4 * 27 * 16 + 27 * 28
# CIC: 4 RK stages x 8 cells x 16 B + post-step 8 x 28 B (+ Jacobian 6 x 27 x 12 B, always TSC)
BYTES_PER_PHOTON_STEP_CIC_NOJAC = 4 * 8 * 16 + 8 * 28
BYTES_PER_PHOTON_STEP_CIC = BYTES_PER_PHOTON_STEP_CIC_NOJAC + 6 * 27 * 12


def catalogue_sources(synth, n, seed, zmax=2.0, half_deg=4.5):
    """Sources uniform in comoving volume inside the cone (octree units), RAMSES-unit velocities."""
    cosmo = synth.Cosmology()
    chi_max = float(cosmo.chi_of_z(zmax)[0]) / 2048.0
    rng = np.random.default_rng(seed)
    d = chi_max * rng.uniform(0.02, 1.0, n) ** (1.0 / 3.0)
    ph = np.radians(rng.uniform(-half_deg, half_deg, n))
    th = np.pi / 2 + np.radians(rng.uniform(-half_deg, half_deg, n))
    src = np.zeros((n, 8))
    src[:, 0] = d * np.cos(ph) * np.sin(th)
    src[:, 1] = d * np.sin(ph) * np.sin(th)
    src[:, 2] = d * np.cos(th)
    src[:, 3:6] = rng.normal(0.0, 1e-3, (n, 3))
    src[:, 6] = np.arange(n)          # id
    src[:, 7] = 1.0                   # npart
    return src


SURR_UNIT = UNIT
# tensor-core work per network evaluation of one point: 4 hidden layers 128x128
# and the output layer 16x128 (multiply-add = 2 FLOP); evaluations per step:
# RK4 stages 2-4 and the post-step point
SURR_FLOP_PER_EVAL = 2 * (4 * 128 * 128 + 16 * 128)
SURR_EVALS_PER_STEP = 4
SURR_TOLERANCE = 1e-3


def surrogate_workload(synth):
    """The uniform 64^3 field (octree level 8) over a 5 x 5 degree cone to z = 2."""
    cosmo = synth.Cosmology()
    chi2 = float(cosmo.chi_of_z(2.0)[0])
    return synth.OctreeSpec(base_level=8, box_cells=64, lbox=2048.0, half_y=2.5, half_z=2.5, chi_max=chi2 * 1.02,
                            halos=0, max_level=8, seed=42), chi2


def measured_peak_bf16():
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


def _deflection_vec(launch, final):
    x = final[:, 2:5]
    return np.cross(launch[:, 3:], x) / np.linalg.norm(x, axis=1)[:, None]


def run_surrogate(args, synth, world, rank, local, dist):
    spec, chi2 = surrogate_workload(synth)
    cos = cosmology_table(synth)
    length = spec.lbox * synth.MPC / spec.cosmo.h
    train_samples = int(args.surrogate_samples)
    config = {"workload": "64^3 periodic field at octree level 8 over a 5x5 deg cone to z=2; 1000x1000 rays; TSC, "
                          "10 steps/cell; surrogate: 64 Fourier frequencies, 4x128 SiLU, 5 outputs, trained on %d "
                          "octree-labelled samples; octree re-check every 64 steps, fallback above %g relative "
                          "deflection drift" % (train_samples, SURR_TOLERANCE),
              "rays": 1000 * 1000, "batch_rays": args.batch, "order": "TSC", "nsteps": 10, "z_stop": 2.0,
              "l2": "inputs and octree re-checks only; the network lives in shared memory",
              "parallelism": "replicas" if world > 1 else "single GPU"}
    kw = dict(nsteps=10, order=2, stop="redshift", stop_value=2.0)
    if args.impl == "reference":
        if rank != 0:
            return
        import oracle as oracle_mod
        oracle_mod.build()
        rec = synth.make_octree(spec)
        launch = ray_grid(1000, 2.5)
        nthreads = os.cpu_count() or 1
        O = oracle_mod.Oracle(rec, {"t": cos[0], "a": cos[1], "dadt": cos[2]}, length, nthreads=nthreads)
        rng = np.random.default_rng(3)
        per_step = 8 * nthreads
        times, counts = [], []
        for k in range(args.warmup + args.steps):
            idx = rng.choice(launch.shape[0], size=per_step, replace=False)
            t0 = time.perf_counter()
            st, _, _ = O.propagate(launch[idx], order=2, nsteps=10, stop="redshift", planes=np.array([2.0]),
                                   jacobian=False)
            dt = time.perf_counter() - t0
            if k >= args.warmup:
                times.append(dt)
                counts.append(int(st.sum()))
        value = sum(counts) / sum(times)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "impl": "reference",
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                                 "sample": "%d random rays per step, C oracle restating the reference's octree "
                                           "path (the reference has no surrogate)" % per_step},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    torch.cuda.set_device(local)
    pkg = importlib.import_module(PKG)
    importlib.import_module(PKG + ".build").build()
    lib = pkg.library()
    capi = importlib.import_module(PKG + ".capi")
    Sur = importlib.import_module(PKG + ".surrogate").Surrogate
    tree = pkg.Octree.from_records(synth.make_octree(spec))
    cosmo = pkg.Cosmology(*cos)
    t = np.tan(np.radians(2.5))
    sur = Sur((t, t), r_max=chi2 * 1.02 / spec.lbox, a_min=1.0 / 3.0 - 0.05, freq_sigma=(6.0, 1.5, 1.5, 0.5),
              seed=42 + rank)
    train = sur.train(tree, samples=train_samples, batch=16384, lr=2e-3)
    launch = ray_grid(1000, 2.5)
    B = min(args.batch, launch.shape[0])
    nb = launch.shape[0] // B
    dev = torch.device("cuda", local)
    replicas = importlib.import_module(PKG + ".replicas")
    d_launch = torch.from_numpy(launch).to(dev)
    d_steps = torch.zeros(B, dtype=torch.int64, device=dev)
    d_final = torch.zeros(B * capi.MPF_PHOTON_FIELDS, dtype=torch.float64, device=dev)
    d_status = torch.zeros(1, dtype=torch.int32, device=dev)
    p, keep = capi.make_params(length, jacobian=False, exact=False, **kw)
    stream = torch.cuda.current_stream(dev)
    plain_ms, plain_steps, sur_s, sur_steps, rel_all, flagged = [], 0, [], 0, [], 0
    whole_s, whole_steps, e2e_t = [], 0, []
    with Clocks(local) as clk:
        for k in range(args.warmup + args.steps):
            off = replicas.batch_ids(k, rank, world, nb) * B
            h = np.ascontiguousarray(launch[off:off + B])
            # plain octree path, device-resident inputs
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            capi.check(lib.mpf_propagate_device(tree._h, cosmo._h, C.byref(p), B, C.c_void_p(d_launch.data_ptr() + off * 48),
                                                C.c_void_p(d_steps.data_ptr()), C.c_void_p(d_final.data_ptr()), None,
                                                C.c_void_p(d_status.data_ptr()), C.c_void_p(stream.cuda_stream)))
            b.record(stream)
            torch.cuda.synchronize()
            ref_final = d_final.view(B, -1).cpu().numpy()
            ref_steps = d_steps.cpu().numpy()
            # surrogate kernel alone (no fallback): speed and measured accuracy
            st, fin, fl, drift, ss = sur.propagate(tree, cosmo, h, length, tolerance=np.inf, fallback=False, **kw)
            # the surrogate form at the tolerance, through the public call (host buffers, fallback included)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            st2, _, fl2, _, ss2 = sur.propagate(tree, cosmo, h, length, tolerance=SURR_TOLERANCE, fallback=True,
                                                want_final=False, **kw)
            e2e = time.perf_counter() - t0
            if k < args.warmup:
                continue
            plain_ms.append(a.elapsed_time(b))
            plain_steps += int((ref_steps - 1).sum())
            sur_s.append(ss["surrogate_seconds"])
            sur_steps += ss["photon_steps"]
            rel_all.append(np.linalg.norm(_deflection_vec(h, fin) - _deflection_vec(h, ref_final), axis=1) /
                           np.linalg.norm(_deflection_vec(h, ref_final), axis=1))
            flagged += int((fl2 & 1).sum())
            delivered = int((st2 - 1).sum())
            whole_s.append(ss2["surrogate_seconds"] + ss2["fallback_seconds"])
            whole_steps += delivered
            e2e_t.append(e2e)
    rel = np.concatenate(rel_all)
    n_rays = B * args.steps
    value = whole_steps / sum(whole_s)
    plain_value = plain_steps / (sum(plain_ms) / 1000.0)
    sur_value = sur_steps / sum(sur_s)
    peak, peak_kind = measured_peak_bf16()
    achieved = sur_value * SURR_EVALS_PER_STEP * SURR_FLOP_PER_EVAL / 1e12
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * sum(whole_s) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 state, bf16 network", "data": "synthetic",
            "config": config,
            "form": "surrogate with octree fallback at %g relative deflection drift" % SURR_TOLERANCE,
            "surrogate": {"kernel_steps_per_s": sur_value, "plain_steps_per_s": plain_value,
                          "kernel_vs_plain": sur_value / plain_value,
                          "flagged_fraction": flagged / n_rays,
                          "rel_deflection_error": {"median": float(np.median(rel)), "p90": float(np.percentile(rel, 90)),
                                                   "max": float(rel.max())},
                          "training": train},
            "e2e": {"value": whole_steps / sum(e2e_t), "unit": UNIT, "h2d_bytes_per_step": B * 6 * 8,
                    "d2h_bytes_per_step": B * (8 + 1 + 4)},
            "gpu_launches": 2 * args.steps,
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                         "traffic": None, "peak_source": peak_kind + " (MEASURED_PEAKS.json bf16_tflops)",
                         "flop_per_photon_step": SURR_EVALS_PER_STEP * SURR_FLOP_PER_EVAL},
            "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)


def surrogate_entry(pkg, synth, capi, lib, rays=131072, samples=50e6):
    """The metric's comparison, measured in the default run: the learned field
    surrogate (BASELINE config 4: the uniform 64^3 field over a 5 x 5 degree
    cone to z = 2, 64 Fourier frequencies, 4 x 128 SiLU, BF16 weights, trained
    on `samples` octree-labelled points) against the plain octree kernel on
    the same rays, with the arithmetic bound of the 5x target."""
    import torch
    spec, chi2 = surrogate_workload(synth)
    cos = cosmology_table(synth)
    length = spec.lbox * synth.MPC / spec.cosmo.h
    Sur = importlib.import_module(PKG + ".surrogate").Surrogate
    tree = pkg.Octree.from_records(synth.make_octree(spec))
    cosmo = pkg.Cosmology(*cos)
    t = np.tan(np.radians(2.5))
    dom = dict(r_max=chi2 * 1.02 / spec.lbox, a_min=1.0 / 3.0 - 0.05, freq_sigma=(6.0, 1.5, 1.5, 0.5))
    sur = Sur((t, t), seed=42, **dom)
    train = sur.train(tree, samples=int(samples), batch=16384, lr=2e-3)
    # the same network untrained (its initial weights, the trained output
    # normalisation): what the training gains
    untrained = Sur((t, t), seed=42, **dom)
    untrained.set_params(None, sur.get_params()[1])
    launch = np.ascontiguousarray(ray_grid(1000, 2.5)[:rays])
    kw = dict(nsteps=10, order=2, stop="redshift", stop_value=2.0)
    # plain octree kernel, device-resident rays, CUDA events on its stream
    dev = torch.device("cuda", torch.cuda.current_device())
    d_launch = torch.from_numpy(launch).to(dev)
    d_steps = torch.zeros(rays, dtype=torch.int64, device=dev)
    d_final = torch.zeros(rays * capi.MPF_PHOTON_FIELDS, dtype=torch.float64, device=dev)
    d_status = torch.zeros(1, dtype=torch.int32, device=dev)
    p, keep = capi.make_params(length, jacobian=False, exact=False, **kw)
    stream = torch.cuda.current_stream(dev)
    plain_ms = []
    for rep in range(3):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        capi.check(lib.mpf_propagate_device(tree._h, cosmo._h, C.byref(p), rays, C.c_void_p(d_launch.data_ptr()),
                                            C.c_void_p(d_steps.data_ptr()), C.c_void_p(d_final.data_ptr()), None,
                                            C.c_void_p(d_status.data_ptr()), C.c_void_p(stream.cuda_stream)))
        b.record(stream)
        torch.cuda.synchronize()
        plain_ms.append(a.elapsed_time(b))
    ref_final = d_final.view(rays, -1).cpu().numpy()
    plain_steps = int((d_steps.cpu().numpy() - 1).sum())
    plain_rate = plain_steps / (min(plain_ms) / 1000.0)
    # the surrogate kernel alone (no re-check fallback): speed and accuracy
    _, fin, _, _, ss = sur.propagate(tree, cosmo, launch, length, tolerance=np.inf, fallback=False, **kw)
    _, fin_u, _, _, _ = untrained.propagate(tree, cosmo, launch, length, tolerance=np.inf, fallback=False, **kw)
    sur_rate = ss["photon_steps"] / ss["surrogate_seconds"]
    # the surrogate form at the tolerance: flagged rays re-run on the octree
    st2, _, fl2, _, ss2 = sur.propagate(tree, cosmo, launch, length, tolerance=SURR_TOLERANCE, fallback=True,
                                        want_final=False, **kw)
    form_rate = int((st2 - 1).sum()) / (ss2["surrogate_seconds"] + ss2["fallback_seconds"])
    ref_d = _deflection_vec(launch, ref_final)

    def rel_err(f):
        r = np.linalg.norm(_deflection_vec(launch, f) - ref_d, axis=1) / np.linalg.norm(ref_d, axis=1)
        return {"median": float(np.median(r)), "p90": float(np.percentile(r, 90)), "max": float(r.max())}

    peak, peak_kind = measured_peak_bf16()
    flop_step = SURR_EVALS_PER_STEP * SURR_FLOP_PER_EVAL
    need = 5.0 * plain_rate * flop_step / 1e12
    out = {"workload": "64^3 uniform field at octree level 8 over a 5x5 deg cone to z=2, %d rays of the 1000x1000 grid, "
                       "TSC, 10 steps/cell; 64 Fourier frequencies, 4x128 SiLU, BF16 weights on the tensor cores, "
                       "trained on %d octree-labelled samples" % (rays, int(samples)),
           "plain_steps_per_s": plain_rate, "surrogate_kernel_steps_per_s": sur_rate,
           "surrogate_form_steps_per_s": form_rate, "form_vs_plain": form_rate / plain_rate,
           "kernel_vs_plain": sur_rate / plain_rate,
           "rel_deflection_error_vs_plain": rel_err(fin), "untrained_rel_deflection_error_vs_plain": rel_err(fin_u),
           "flagged_fraction_at_tolerance": float((fl2 & 1).mean()), "tolerance": SURR_TOLERANCE,
           "mma_tflops": sur_rate * flop_step / 1e12,
           "bound_of_5x": {"flop_per_photon_step": flop_step, "tflops_needed": need, "bf16_peak_tflops": peak,
                           "peak_source": peak_kind, "needed_over_peak": need / peak},
           "training": train}
    for o in (sur, untrained, tree, cosmo):
        o.close()
    del keep
    return out


MAPS_METRIC = "HEALPix map photon-steps/s (mpf_hmaps_fill: kappa, gamma1, gamma2, 1/mu, nside 4096, one full-sky cone)"
MAPS_HALF_DEG = 14.7   # a square cone of (2 x 14.7 deg)^2 = 0.263 sr: 1/48 of the sky


def maps_cone_spec(synth):
    """One of the 48 full-sky cones of BASELINE config 5: the 512^3 periodic
    base (octree level 11, file level 9) over lbox = 2048 Mpc/h, refined to
    level 14 in this cone's 417 of the 20 000 NFW haloes, to z = 1."""
    cosmo = synth.Cosmology()
    chi1 = float(cosmo.chi_of_z(1.0)[0])
    return synth.OctreeSpec(base_level=11, box_cells=512, lbox=2048.0, half_y=MAPS_HALF_DEG, half_z=MAPS_HALF_DEG,
                            chi_max=chi1 * 1.02, halos=417, max_level=14, mass_min=1e12, mass_max=1e15,
                            refine_cells=4.5, seed=48)


def maps_cone_pixels(pkg, nside):
    """The RING pixels of nside whose centres lie in the square cone about +x
    (|phi| and |theta - 90 deg| at most MAPS_HALF_DEG): candidates from the
    equatorial rings near phi = 0, centres from the library's pix2vec_ring."""
    t = np.sin(np.radians(MAPS_HALF_DEG)) * 1.01
    # equatorial rings i (nside <= i <= 3 nside) have z = 4/3 - 2 i / (3 nside), 4 nside pixels each
    i_lo = int(np.floor((4.0 / 3.0 - t) * 1.5 * nside)) - 1
    i_hi = int(np.ceil((4.0 / 3.0 + t) * 1.5 * nside)) + 1
    rings = np.arange(max(i_lo, nside), min(i_hi, 3 * nside) + 1)
    jmax = int(np.ceil(np.radians(MAPS_HALF_DEG) / (np.pi / (2 * nside)))) + 2
    j = np.concatenate([np.arange(0, jmax + 1), np.arange(4 * nside - jmax - 1, 4 * nside)])
    cand = (2 * nside * (nside - 1) + 4 * nside * (rings[:, None] - nside) + j[None, :]).ravel()
    v = pkg.pix2vec_ring(nside, cand)
    ph = np.degrees(np.arctan2(v[:, 1], v[:, 0]))
    th = np.degrees(np.arccos(np.clip(v[:, 2], -1.0, 1.0)))
    keep = (np.abs(ph) <= MAPS_HALF_DEG) & (np.abs(th - 90.0) <= MAPS_HALF_DEG)
    return np.sort(cand[keep]), v[keep][np.argsort(cand[keep])]


def run_maps(args, synth, world, rank, local, dist):
    """BASELINE config 5 on one full-sky cone: the octree built on the GPU from
    the reference's 10-column ASCII cell rows (mpf_cells_build, timed), then
    the kappa / gamma / 1/mu maps of its nside = 4096 pixels to z_s = 1
    (mpf_hmaps_fill, TSC, 8 steps per cell); a step = one call on a chunk of
    the cone's pixels.  Photon-steps are read from the maps' steps row: the
    trajectory index before the z_s = 1 crossing, where the ray stops, plus
    one (a ray that leaves the data first has a zero row and is not
    counted).  The FLRW values of the surface are not read by these rows."""
    spec = maps_cone_spec(synth)
    cos = cosmology_table(synth)
    length = spec.lbox * synth.MPC / spec.cosmo.h
    nside = 4096
    chunk = args.batch
    comps = ["lensing", "steps"]
    config = {"workload": "one of 48 full-sky cones (a (2 x 14.7 deg)^2 square, 0.263 sr) of a 512^3 periodic field at "
                          "octree level 11 (lbox 2048 Mpc/h) refined to level 14 in 417 NFW haloes, to z_s=1; HEALPix "
                          "nside 4096 RING pixel centres of the cone, one ray each; TSC, 8 steps/cell, infinitesimal "
                          "Jacobian; octree built on the GPU from the 10-column ASCII cell rows",
              "nside": nside, "pixels_per_step": chunk, "order": "TSC", "nsteps": 8, "z_s": 1.0,
              "gather_arithmetic": "fp32 gather, fp64 state", "maps": "kappa gamma1 gamma2 1/mu steps (float)",
              "l2": "octree larger than L2 (no flush)", "parallelism": "single GPU"}
    key = hashlib.sha1(repr(spec).encode()).hexdigest()[:16]
    path = os.path.join(os.environ.get("TMPDIR", "/tmp"), "mpf_bench_%s.bin" % key)
    t0 = time.perf_counter()
    if os.path.exists(path):
        rec0 = synth.read_bin(path)
    else:
        rec0 = synth.make_octree(spec)
        synth.write_bin(path + ".tmp", rec0)
        os.replace(path + ".tmp", path)
    gen_s = time.perf_counter() - t0
    rows = synth.cells_ramses(rec0, spec).astype(np.float32)
    if args.impl == "reference":
        if rank != 0:
            return
        import oracle as oracle_mod
        oracle_mod.build()
        nthreads = os.cpu_count() or 1
        O = oracle_mod.Oracle(rec0, {"t": cos[0], "a": cos[1], "dadt": cos[2]}, length, nthreads=nthreads)
        pk = importlib.import_module(PKG)
        _, dirs = maps_cone_pixels(pk, nside)
        rng = np.random.default_rng(3)
        times, counts = [], []
        for k in range(args.warmup + args.steps):
            idx = rng.choice(dirs.shape[0], size=2 * nthreads, replace=False)
            launch = np.zeros((idx.shape[0], 6))
            launch[:, 3:] = dirs[idx]
            t1 = time.perf_counter()
            st, _, _ = O.propagate(launch, order=2, nsteps=8, stop="redshift", planes=np.array([1.0]), jacobian=True)
            dt = time.perf_counter() - t1
            if k >= args.warmup:
                times.append(dt)
                counts.append(int(st.sum()))
        value = sum(counts) / sum(times)
        print(json.dumps({"metric": MAPS_METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                          "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times), "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                          "impl": "reference",
                          "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                                           "sample": "%d random pixels per step, C oracle (trajectory then Jacobian)"
                                                     % (2 * nthreads)},
                          "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
              flush=True)
        return
    import torch
    torch.cuda.set_device(local)
    pkg = importlib.import_module(PKG)
    importlib.import_module(PKG + ".build").build()
    capi = importlib.import_module(PKG + ".capi")
    cosmo = pkg.Cosmology(*cos)
    # the octree build on the GPU from the ASCII rows (importascii + correctOctree)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    built = pkg.cells_build(rows, cosmo, (0.0, 0.0, 0.0), (spec.chi_max / spec.lbox, 0.0, 0.0),
                            np.arctan(np.sqrt(2.0) * np.tan(np.radians(MAPS_HALF_DEG))) * 1.02, (0.0, 0.0, 0.0),
                            4.0 / 512.0, spec.cosmo.h, spec.cosmo.omega_m, spec.lbox, synth.MPC, order=2)
    build_s = time.perf_counter() - t0
    completion = pkg.cells_completion_info()
    built = np.frombuffer(built.tobytes(), dtype=synth.RECORD)
    t0 = time.perf_counter()
    tree = pkg.Octree.from_records(built)
    upload_s = time.perf_counter() - t0
    info = tree.info
    pixels, dirs = maps_cone_pixels(pkg, nside)
    nb = max(1, pixels.shape[0] // chunk)
    config.update({"cells": int(info["cells"]), "levels": [info["level_min"], info["level_max"]],
                   "octree_device_bytes": int(info["device_bytes"]), "cone_pixels": int(pixels.shape[0]),
                   "ascii_rows": int(rows.shape[0])})
    cz = cosmo_mod_homogeneous(synth, cos, [1.0])
    p, keep = capi.make_params(length, 8, 2, "redshift", 0.0, np.array([1.0]), True, args.exact, 0)
    kw = dict(nsteps=8, order=2, exact=args.exact)

    def call(k):
        px = np.ascontiguousarray(pixels[(k % nb) * chunk:(k % nb + 1) * chunk])
        return pkg.hmaps_fill(tree, cosmo, nside, px, np.array([1.0]), cz, comps, length, **kw)

    for k in range(args.warmup):
        call(k)
    torch.cuda.synchronize()
    steps_total, t_calls = 0, []
    with Clocks(local) as clk:
        for k in range(args.steps):
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            m = call(args.warmup + k)
            t_calls.append(time.perf_counter() - t1)
            fid = m[0, 4].astype(np.float64)
            steps_total += int((fid + (fid > 0)).sum())   # a ray stopped at z_s: its steps are firstid + 1
    value = steps_total / sum(t_calls)
    # map-level error against the float64 (reference-order) kernel on a pixel sample
    rng = np.random.default_rng(5)
    sample = np.sort(rng.choice(pixels, size=min(2048, pixels.shape[0]), replace=False))
    fast = pkg.hmaps_fill(tree, cosmo, nside, sample, np.array([1.0]), cz, comps, length, nsteps=8, order=2, exact=False)
    exact = pkg.hmaps_fill(tree, cosmo, nside, sample, np.array([1.0]), cz, comps, length, nsteps=8, order=2, exact=True)
    map_err = {}
    for r, name in enumerate(("kappa", "gamma1", "gamma2", "inv_mu")):
        e, sc = np.abs(fast[0, r] - exact[0, r]).max(), np.abs(exact[0, r]).max()
        map_err[name] = {"abs_max": float(e), "scale": float(sc), "of_scale": float(e / max(sc, 1e-30))}
    map_err["steps_rows_equal"] = bool(np.array_equal(fast[0, 4], exact[0, 4]))
    map_err["sample_pixels"] = int(sample.shape[0])
    peak, peak_kind = measured_peak_hbm()
    achieved = value * BYTES_PER_PHOTON_STEP / 1e9
    line = {"metric": MAPS_METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * sum(t_calls) / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": chunk * 8,
                    "d2h_bytes_per_step": chunk * 5 * 4},
            "build": {"synthetic_field_s": gen_s, "cells_build_s": build_s, "octree_upload_s": upload_s,
                      "ascii_rows": int(rows.shape[0]), "cells": int(info["cells"]), "completion": completion},
            "map_error_vs_float64_kernel": map_err,
            "gpu_launches": 3 * args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "peak_source": peak_kind, "bytes_per_photon_step": BYTES_PER_PHOTON_STEP,
                         "scope": "whole mpf_hmaps_fill call (host pixels in, float maps out)"},
            "clocks": clk.summary()}
    del keep
    if rank == 0:
        print(json.dumps(line), flush=True)


def cosmo_mod_homogeneous(synth, cos, zs):
    """FillMap's per-surface FLRW values (t, chi, lambda, a, z) at redshift
    surfaces, from the cosmology table: a = 1 / (1 + z), t and chi = c t / L
    read off the table (the homogeneous ray's lambda is t for dt/dl = 1)."""
    t, a = cos[0], cos[1]
    out = np.zeros((len(zs), 5))
    for k, z in enumerate(zs):
        ak = 1.0 / (1.0 + z)
        tk = float(np.interp(-ak, -a, t))
        chi = float(synth.Cosmology().chi_of_z(z)[0]) / 2048.0
        out[k] = (tk, chi, tk, ak, z)
    return out


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("MPF_BENCH_GLOO") is None else "gloo")
    return world, rank, local, dist


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=None,
                    help="rays (maps: pixels) per step; default: the whole 1000x1000 grid in one batch for the "
                         "propagation line (the persistent launch's tail of long rays is a smaller share of a larger "
                         "batch: 8.05e8 photon-steps/s at 250000 rays, 8.83e8 at 500000, 8.86e8 at 1000000), 250000 "
                         "for the other modes")
    ap.add_argument("--workload", default="amr", choices=["amr", "medium", "small", "cones16"],
                    help="amr = the benchmark configuration; cones16 = the catalogue over 16 cones of the uniform "
                         "64^3 field (with --mode catalogue); medium / small for profiling and debugging")
    ap.add_argument("--exact", action="store_true", help="reference float64 gather order")
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU baseline, the parity object and the accuracy statistic (profiling runs)")
    ap.add_argument("--zstop", type=float, default=2.0, help="stop redshift (profiling captures use a short path)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-catalogue", action="store_true",
                    help="leave the catalogue root-finder's sub-object out of the default line")
    ap.add_argument("--no-surrogate", action="store_true",
                    help="skip the surrogate-vs-plain comparison of the default line")
    ap.add_argument("--mode", default="propagate", choices=["propagate", "catalogue", "surrogate", "maps", "velocity"],
                    help="propagate = the headline ray-tracing benchmark; catalogue = the Newton root-finder; "
                         "surrogate = the learned field in the RK4 stages against the plain octree; maps = HEALPix "
                         "lensing maps of one full-sky cone at nside 4096; velocity = the velocity-field "
                         "deposit and the Doppler-redshift trace")
    ap.add_argument("--particles", type=int, default=1 << 24, help="particles of the velocity-field deposit")
    ap.add_argument("--surrogate-samples", type=float, default=50e6, help="training samples of the surrogate")
    ap.add_argument("--sources", type=int, default=262144,
                    help="catalogue sources per step (a call's rounds wait for its slowest sources, whose up to 11 "
                         "sequential rays cross halo cores; 2^18 sources amortise that chain)")
    args = ap.parse_args()
    if args.batch is None:
        args.batch = 1000 * 1000 if args.mode == "propagate" and not args.exact else 250000
    world, rank, local, dist = dist_setup()
    synth = importlib.import_module(PKG + ".synth")
    spec = workload_spec(synth, args.workload)
    config = {"workload": "AMR cone octree, 256^3 base (level 10) refined to level 14 in 2000 NFW haloes; "
                          "1000x1000 rays over 10x10 deg to z=2; TSC, 8 steps/cell, infinitesimal Jacobian at z=2"
                          if args.workload == "amr" else "%s octree (profiling / debugging)" % args.workload,
              "rays": 1000 * 1000, "batch_rays": args.batch, "order": "TSC", "nsteps": 8, "z_stop": args.zstop,
              "gather_arithmetic": "float64 reference order" if args.exact else "fp32 gather, fp64 state",
              "streams": "steps alternate between 2 CUDA streams (a batch's tail overlaps the next batch)",
              "l2": "octree larger than L2 (no flush)", "parallelism": "replicas" if world > 1 else "single GPU"}
    cos = cosmology_table(synth)
    length = spec.lbox * synth.MPC / spec.cosmo.h
    planes = np.array([args.zstop])
    if args.mode == "catalogue":
        return run_catalogue(args, synth, spec, cos, length, world, rank, local, dist)
    if args.mode == "surrogate":
        return run_surrogate(args, synth, world, rank, local, dist)
    if args.mode == "maps":
        return run_maps(args, synth, world, rank, local, dist)
    if args.mode == "velocity":
        return run_velocity(args, synth, spec, cos, length, world, rank, local, dist)

    if args.impl == "reference":
        if rank != 0:
            return
        import oracle as oracle_mod
        oracle_mod.build()
        rec = octree_records(synth, spec)
        launch = ray_grid()
        nthreads = os.cpu_count() or 1
        O = oracle_mod.Oracle(rec, {"t": cos[0], "a": cos[1], "dadt": cos[2]}, length, nthreads=nthreads)
        rng = np.random.default_rng(3)
        per_step = 2 * nthreads
        times, counts = [], []
        for s in range(args.warmup + args.steps):
            idx = rng.choice(launch.shape[0], size=per_step, replace=False)
            t0 = time.perf_counter()
            st, _, _ = O.propagate(launch[idx], order=2, nsteps=8, stop="redshift", planes=planes, jacobian=True)
            dt = time.perf_counter() - t0
            if s >= args.warmup:
                times.append(dt)
                counts.append(int(st.sum()))
        value = sum(counts) / sum(times)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "impl": "reference",
                "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                                 "sample": "%d random rays per step of the grid, C oracle restating the reference "
                                           "(the reference's x86 build does not run on this Arm host)" % per_step},
                "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    torch.cuda.set_device(local)
    pkg = importlib.import_module(PKG)
    importlib.import_module(PKG + ".build").build()
    lib = pkg.library()
    capi = importlib.import_module(PKG + ".capi")
    rec = octree_records(synth, spec)
    tree = pkg.Octree.from_records(rec)
    info = tree.info
    config.update({"cells": int(info["cells"]), "levels": [info["level_min"], info["level_max"]],
                   "octree_device_bytes": int(info["device_bytes"])})
    cosmo = pkg.Cosmology(*cos)
    launch = ray_grid()
    B = min(args.batch, launch.shape[0])
    # batches of B rays over the whole grid, the last one shorter
    nb = -(-launch.shape[0] // B)
    config["batches"] = "%d of %d rays and one of %d, in turn" % (nb - 1, B, launch.shape[0] - (nb - 1) * B) \
        if launch.shape[0] % B else ("%d of %d rays, in turn" % (nb, B) if nb > 1 else
                                     "the whole grid, one launch per step")
    dev = torch.device("cuda", local)
    d_launch = torch.from_numpy(launch).to(dev)
    d_steps = torch.zeros((args.warmup + args.steps, B), dtype=torch.int64, device=dev)
    # two streams: step k runs on streams[k % 2] with its own output buffer, so
    # a batch's last long rays overlap the start of the next batch instead of
    # leaving SMs idle (the map driver gets the same from its 4M-pixel launches)
    streams = [torch.cuda.current_stream(dev), torch.cuda.Stream(dev)]
    d_planes = [torch.zeros(B * 1 * capi.MPF_PLANE_FIELDS, dtype=torch.float64, device=dev) for _ in streams]
    d_status = torch.zeros(1, dtype=torch.int32, device=dev)
    p, keep = capi.make_params(length, nsteps=8, order=2, stop="redshift", planes=planes, jacobian=True,
                               exact=args.exact)
    stream = streams[0]

    replicas = importlib.import_module(PKG + ".replicas")

    def step(k):
        off = replicas.batch_ids(k, rank, world, nb) * B
        size = min(B, launch.shape[0] - off)
        rc = lib.mpf_propagate_device(tree._h, cosmo._h, C.byref(p), size, C.c_void_p(d_launch.data_ptr() + off * 48),
                                      C.c_void_p(d_steps[k].data_ptr()), None, C.c_void_p(d_planes[k % 2].data_ptr()),
                                      C.c_void_p(d_status.data_ptr()), C.c_void_p(streams[k % 2].cuda_stream))
        capi.check(rc)

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        ev0.record(stream)
        streams[1].wait_event(ev0)
        for k in range(args.steps):
            step(args.warmup + k)
        stream.wait_stream(streams[1])
        ev1.record(stream)
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    elapsed_ms = ev0.elapsed_time(ev1)
    photon_steps = int(d_steps[args.warmup:].sum().item())
    status = int(d_status.item())
    t_max, total_steps = replicas.reduce_counters(dist, elapsed_ms, photon_steps, dev)
    value = total_steps / (t_max / 1000.0)

    # end to end through the public API: host launch records in, host steps and
    # surface records out, every step
    e2e_t = []
    e2e_steps = 0
    for k in range(0 if args.no_e2e else max(2, min(args.steps, 3))):
        off = ((k + 1) % nb) * B
        h = np.ascontiguousarray(launch[off:off + B])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st, _, pl, _ = pkg.propagate(tree, cosmo, h, length, nsteps=8, order=2, stop="redshift", planes=planes,
                                     jacobian=True, exact=args.exact, want_final=False)
        e2e_t.append(time.perf_counter() - t0)
        e2e_steps += int(st.sum())
    e2e_value = e2e_steps / sum(e2e_t) if e2e_t else None

    peak, peak_kind = measured_peak_hbm()
    # consecutive launches overlap (two streams): a launch's share of the
    # timed region is its duration
    avg_launch_s = (elapsed_ms / args.steps) / 1000.0
    bytes_per_launch = (photon_steps / args.steps) * BYTES_PER_PHOTON_STEP
    achieved = bytes_per_launch / avg_launch_s / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": (DRAM_BYTES_PER_PHOTON_STEP * photon_steps / args.steps) if DRAM_BYTES_PER_PHOTON_STEP else None,
                "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured" else peak_kind,
                "bytes_per_photon_step": BYTES_PER_PHOTON_STEP}
    clk_summary = clk.summary()
    roofline["fp64"] = fp64_roofline(value / world, clk_summary)
    tuned = pkg.autotune_info(tree, "propagate", 2)
    config["autotune"] = ({"threads_per_block": tuned[0], "rays_per_lane_per_claim": tuned[1],
                           "candidates_photon_steps_per_s": dict(zip(("128x1", "64x1", "32x1", "128x2"), tuned[2]))}
                          if tuned else None)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
            "form": "plain octree (the surrogate form against it: the surrogate entry)",
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": B * 6 * 8,
                    "d2h_bytes_per_step": B * 8 + B * capi.MPF_PLANE_FIELDS * 8},
            "gpu_launches": args.steps, "roofline": roofline, "status_bits": status,
            "clocks": clk_summary}
    if rank == 0 and not args.no_cpu_baseline:
        import oracle as oracle_mod
        oracle_mod.build()
        line["cpu_baseline"], oracle_run = cpu_baseline(oracle_mod, rec, cos, length, launch, planes)
        line["parity"] = parity_entry(pkg, tree, cosmo, length, planes, oracle_run, exact=args.exact)
    if rank == 0 and not args.exact and not args.no_cpu_baseline:
        # the library's own statement of the call's error (mpf_propagate_accuracy): the same
        # kernel against the float64 kernel on 256 rays spread over the grid
        acc = pkg.propagate_accuracy(tree, cosmo, launch, length, sample=256, nsteps=8, order=2, stop="redshift",
                                     planes=planes, jacobian=True)
        acc["against"] = "the float64 kernel (the reference's operation order), mpf_propagate_accuracy"
        line["accuracy_of_call"] = acc
    if rank == 0 and not args.no_catalogue:
        line["catalogue"] = catalogue_entry(pkg, capi, lib, synth, tree, cosmo, length, spec.cosmo.h, dev)
    if rank == 0 and not args.no_surrogate:
        tree.close()      # the benchmark octree's 5 GB are not needed any more
        line["surrogate"] = surrogate_entry(pkg, synth, capi, lib)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def catalogue_entry(pkg, capi, lib, synth, tree, cosmo, length, h, dev, nsrc=262144, calls=2):
    """The catalogue root-finder (Catalogues::relCat's Newton iterations) on
    the benchmark octree, in the default line: nsrc sources uniform in
    comoving volume to z = 2 inside 9 x 9 deg, cat_accuracy 1e-8, TSC,
    8 steps per cell; one warm-up call, then `calls` calls of
    mpf_catalogue_newton_device on one stream (sources resident on the
    device), timed with CUDA events.  `--mode catalogue` measures the same
    workload with two host threads alternating their calls."""
    import torch
    kw = dict(cat_accuracy=1e-8, nsteps=8, order=2, vobs=(0.0, 0.0, 0.0), max_iterations=10)
    pool = catalogue_sources(synth, nsrc * (calls + 1), 17)
    d_src = torch.from_numpy(pool).to(dev)
    d_rows = torch.zeros((nsrc, capi.MPF_CATALOGUE_FIELDS), dtype=torch.float64, device=dev)
    p, keep = pkg.catalogue_params(length, h, **kw)
    stream = torch.cuda.current_stream(dev)
    stats = []

    def call(k):
        st = capi.CatalogueStats()
        capi.check(lib.mpf_catalogue_newton_device(tree._h, cosmo._h, C.byref(p), nsrc,
                                                   C.c_void_p(d_src.data_ptr() + k * nsrc * 8 * 8), 8,
                                                   C.c_void_p(d_rows.data_ptr()), C.byref(st),
                                                   C.c_void_p(stream.cuda_stream)))
        return pkg.catalogue_stats(st)

    call(0)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for k in range(1, calls + 1):
        stats.append(call(k))
    ev1.record(stream)
    torch.cuda.synchronize()
    sec = ev0.elapsed_time(ev1) / 1000.0
    rows = d_rows.cpu().numpy()
    del keep
    return {"metric": CAT_METRIC, "value": nsrc * calls / sec, "unit": CAT_UNIT, "sources_per_call": nsrc,
            "calls": calls, "ms_per_call": 1000.0 * sec / calls,
            "photon_steps_per_s": sum(s["photon_steps"] for s in stats) / sec,
            "rays_per_source": sum(s["rays"] for s in stats) / (nsrc * calls),
            "converged_fraction": float(np.mean((rows[:, 2] != 42) & (rows[:, 5] != 42))),
            "gpu_launches": sum(s["kernel_launches"] for s in stats),
            "workload": "%d sources per call uniform in comoving volume to z=2 inside 9x9 deg on the benchmark "
                        "octree, cat_accuracy 1e-8, TSC, 8 steps/cell; one stream, sources on the device" % nsrc}


# 16 narrow cones over the 64^3 uniform field (octree level 8) to z = 2, the
# cones' axes on a 4 x 4 grid of narrow-cone angles (phi, theta)
CONES16_AXES = [(p, t) for p in (-45.0, -15.0, 15.0, 45.0) for t in (-45.0, -15.0, 15.0, 45.0)]


def cones16_records(synth):
    """One octree shared by the 16 cones: the union of the cones' cells (the
    field of a cell depends only on its key, so shared cells agree)."""
    key = "cones16_v1"
    path = os.path.join(os.environ.get("TMPDIR", "/tmp"), "mpf_bench_%s.bin" % key)
    if os.path.exists(path):
        return synth.read_bin(path)
    parts = [synth.make_octree(synth.uniform_grid_cone(2.0, ax)) for ax in CONES16_AXES]
    rec = np.concatenate(parts)
    order = np.lexsort((rec["lo"], rec["hi"]))
    rec = rec[order]
    keep = np.ones(rec.shape[0], dtype=bool)
    keep[1:] = (rec["hi"][1:] != rec["hi"][:-1]) | (rec["lo"][1:] != rec["lo"][:-1])
    rec = rec[keep]
    tmp = path + ".%d" % os.getpid()
    synth.write_bin(tmp, rec)
    os.replace(tmp, path)
    return rec


def cones16_sources(synth, n, seed, zmin=0.05, zmax=2.0, half_deg=2.4):
    """Sources uniform in the light-cone volume between zmin and zmax, spread
    evenly over the 16 cones (square 2 half_deg cones about their axes)."""
    cosmo = synth.Cosmology()
    c0, c1 = (float(cosmo.chi_of_z(z)[0]) / 2048.0 for z in (zmin, zmax))
    rng = np.random.default_rng(seed)
    d = (c0 ** 3 + (c1 ** 3 - c0 ** 3) * rng.random(n)) ** (1.0 / 3.0)
    ph = np.radians(rng.uniform(-half_deg, half_deg, n))
    th = np.pi / 2 + np.radians(rng.uniform(-half_deg, half_deg, n))
    local = np.stack([np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th)], axis=1)
    cone = np.arange(n) % len(CONES16_AXES)
    frames = np.stack([synth.cone_frame(*ax) for ax in CONES16_AXES])
    dirs = np.einsum("nij,nj->ni", frames[cone], local)
    src = np.zeros((n, 8))
    src[:, 0:3] = dirs * d[:, None]
    src[:, 3:6] = rng.normal(0.0, 1e-3, (n, 3))
    src[:, 6] = np.arange(n)
    src[:, 7] = 1.0
    return src


def run_catalogue(args, synth, spec, cos, length, world, rank, local, dist):
    h = spec.cosmo.h
    cones16 = args.workload == "cones16"
    if cones16:
        workload = ("catalogue over 16 narrow cones of the 64^3 uniform field at octree level 8 (file level 6), axes "
                    "phi, theta in {-45,-15,15,45} deg, one shared octree to z=2: %d sources per step uniform in the "
                    "light-cone volume between z=0.05 and z=2 (path lengths up to 24x apart), all 16 cones in each "
                    "call, cat_accuracy 1e-8, CIC, 10 steps/cell" % args.sources)
    elif args.workload == "amr":
        workload = ("catalogue on the AMR cone octree (256^3 base refined to level 14 in 2000 NFW haloes): "
                    "%d sources per step uniform in comoving volume to z=2 inside 9x9 deg, cat_accuracy 1e-8, "
                    "TSC, 8 steps/cell" % args.sources)
    else:
        workload = "catalogue on the %s octree (profiling / debugging)" % args.workload
    config = {"workload": workload, "sources_per_step": args.sources,
              "streams": "steps alternate between 2 host threads / CUDA streams", "order": "CIC" if cones16 else "TSC",
              "nsteps": 10 if cones16 else 8, "cat_accuracy": 1e-8, "max_rays_per_source": 11,
              "gather_arithmetic": "float64 reference order" if args.exact else "fp32 gather, fp64 state",
              "execution": "one CUDA graph launch per call: set-up, sort, one persistent kernel on a device work queue"
                           if not args.exact else "one ray launch per Newton round",
              "l2": "octree smaller than L2 (the 16 cones of a 64^3 field)" if cones16 else "octree larger than L2 (no flush)",
              "parallelism": "replicas" if world > 1 else "single GPU"}
    kw = dict(cat_accuracy=1e-8, nsteps=10 if cones16 else 8, order=1 if cones16 else 2, vobs=(0.0, 0.0, 0.0),
              max_iterations=10)
    nsrc = args.sources

    def records():
        return cones16_records(synth) if cones16 else octree_records(synth, spec)

    def make_sources(count, seed):
        return cones16_sources(synth, count, seed) if cones16 else catalogue_sources(synth, count, seed)
    if args.impl == "reference":
        if rank != 0:
            return
        import oracle as oracle_mod
        oracle_mod.build()
        rec = records()
        nthreads = os.cpu_count() or 1
        O = oracle_mod.Oracle(rec, {"t": cos[0], "a": cos[1], "dadt": cos[2]}, length, nthreads=nthreads)
        per_step = nthreads
        times, counts = [], 0
        for s in range(args.warmup + args.steps):
            src = make_sources(per_step, 1000 + s)
            t0 = time.perf_counter()
            O.catalogue(src, h=h, **kw)
            dt = time.perf_counter() - t0
            if s >= args.warmup:
                times.append(dt)
                counts += per_step
        value = counts / sum(times)
        line = {"metric": CAT_METRIC, "value": value, "unit": CAT_UNIT, "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000 * sum(times) / len(times), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
                "impl": "reference",
                "cpu_baseline": {"value": value, "unit": CAT_UNIT, "cores": nthreads, "kind": "port",
                                 "sample": "%d sources per step, C oracle restating iterateNewtonMethod" % per_step},
                "e2e": {"value": value, "unit": CAT_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    import torch
    torch.cuda.set_device(local)
    pkg = importlib.import_module(PKG)
    importlib.import_module(PKG + ".build").build()
    lib = pkg.library()
    capi = importlib.import_module(PKG + ".capi")
    rec = records()
    tree = pkg.Octree.from_records(rec)
    info = tree.info
    config.update({"cells": int(info["cells"]), "levels": [info["level_min"], info["level_max"]]})
    cosmo = pkg.Cosmology(*cos)
    dev = torch.device("cuda", local)
    nstep = args.warmup + args.steps
    pool = make_sources(nsrc * nstep, 7 + rank)
    d_src = torch.from_numpy(pool).to(dev)
    # two host threads, each with its own stream and rows, take the steps in
    # turn: the Newton rounds of one call wait on host syncs and end with a
    # few slow sources, and the other call's rays fill the GPU meanwhile
    streams = [torch.cuda.current_stream(dev), torch.cuda.Stream(dev)]
    d_rows_s = [torch.zeros((nsrc, capi.MPF_CATALOGUE_FIELDS), dtype=torch.float64, device=dev) for _ in streams]
    d_rows = d_rows_s[0]
    p, keep = pkg.catalogue_params(length, h, exact=args.exact, **kw)
    stream = streams[0]
    stats = []

    def step(k, j=0):
        st = capi.CatalogueStats()
        rc = lib.mpf_catalogue_newton_device(tree._h, cosmo._h, C.byref(p), nsrc,
                                             C.c_void_p(d_src.data_ptr() + k * nsrc * 8 * 8), 8,
                                             C.c_void_p(d_rows_s[j].data_ptr()), C.byref(st),
                                             C.c_void_p(streams[j].cuda_stream))
        capi.check(rc)
        return pkg.catalogue_stats(st)

    def lane(j, ks, out):
        torch.cuda.set_device(local)
        for k in ks:
            out.append(step(k, j))

    for k in range(args.warmup):
        step(k)
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    import threading
    with Clocks(local) as clk:
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        streams[1].wait_event(ev0)
        outs = [[], []]
        lanes = [threading.Thread(target=lane, args=(j, range(args.warmup + j, args.warmup + args.steps, 2), outs[j]))
                 for j in range(2)]
        for t in lanes:
            t.start()
        for t in lanes:
            t.join()
        if len(outs[0]) + len(outs[1]) != args.steps:
            raise RuntimeError("a catalogue lane failed")
        stats.extend(outs[0] + outs[1])
        stream.wait_stream(streams[1])
        ev1.record(stream)
        torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    elapsed_ms = ev0.elapsed_time(ev1)
    replicas = importlib.import_module(PKG + ".replicas")
    t_max, total_src = replicas.reduce_counters(dist, elapsed_ms, nsrc * args.steps, dev)
    value = total_src / (t_max / 1000.0)
    psteps = sum(s["photon_steps"] for s in stats)
    psteps_jac = sum(s["photon_steps_jacobian"] for s in stats)
    rays = sum(s["rays"] for s in stats)
    rows = d_rows.cpu().numpy()
    converged = float(np.mean((rows[:, 2] != 42) & (rows[:, 5] != 42)))

    e2e_t, e2e_n = [], 0
    for k in range(0 if args.no_e2e else 2):
        hsrc = np.ascontiguousarray(pool[k * nsrc:(k + 1) * nsrc])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pkg.catalogue(tree, cosmo, hsrc, length, h, exact=args.exact, **kw)
        e2e_t.append(time.perf_counter() - t0)
        e2e_n += nsrc
    e2e_value = e2e_n / sum(e2e_t) if e2e_t else None

    peak, peak_kind = measured_peak_hbm()
    avg_s = (elapsed_ms / args.steps) / 1000.0   # the calls overlap: each one's share of the timed region
    b_jac, b_nojac = (BYTES_PER_PHOTON_STEP_CIC, BYTES_PER_PHOTON_STEP_CIC_NOJAC) if cones16 else \
        (BYTES_PER_PHOTON_STEP, BYTES_PER_PHOTON_STEP_NOJAC)
    alg_bytes = (b_nojac * (psteps - psteps_jac) + b_jac * psteps_jac) / args.steps
    achieved = alg_bytes / avg_s / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": (DRAM_BYTES_PER_PHOTON_STEP * psteps / args.steps) if DRAM_BYTES_PER_PHOTON_STEP and not cones16
                else None,
                "peak_source": peak_kind, "scope": "whole mpf_catalogue_newton_device call (set-up, sort, persistent kernel)",
                "bytes_per_photon_step": {"with_jacobian": b_jac, "without_jacobian": b_nojac}}
    tuned = pkg.autotune_info(tree, "catalogue", kw["order"])
    config["autotune"] = ({"threads_per_block": tuned[0], "candidates_photon_steps_per_s": {"128": tuned[2][0],
                           "64": tuned[2][1], "32": tuned[2][2]}} if tuned else None)
    line = {"metric": CAT_METRIC, "value": value, "unit": CAT_UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
            "photon_steps_per_s": psteps * world / (t_max / 1000.0), "rays_per_source": rays / (nsrc * args.steps),
            "converged_fraction": converged,
            "e2e": {"value": e2e_value, "unit": CAT_UNIT, "h2d_bytes_per_step": nsrc * 8 * 8,
                    "d2h_bytes_per_step": nsrc * capi.MPF_CATALOGUE_FIELDS * 8},
            "gpu_launches": sum(s["kernel_launches"] for s in stats), "roofline": roofline, "clocks": clk.summary()}
    if rank == 0 and not args.no_cpu_baseline:
        import oracle as oracle_mod
        oracle_mod.build()
        nthreads = os.cpu_count() or 1
        O = oracle_mod.Oracle(rec, {"t": cos[0], "a": cos[1], "dadt": cos[2]}, length, nthreads=nthreads)
        src = make_sources(2 * nthreads, 99)
        t0 = time.perf_counter()
        O.catalogue(src, h=h, **kw)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": src.shape[0] / dt, "unit": CAT_UNIT, "cores": nthreads, "kind": "port",
                                "sample": "%d sources, %.1f s, %d threads (C oracle restating iterateNewtonMethod)"
                                          % (src.shape[0], dt, nthreads)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()




VEL_METRIC = "velocity-field deposit particles/s (TSC onto every level of the AMR cone octree, reference order)"
VEL_UNIT = "particles/s"
VEL_VOBS = (3e-4, -2e-4, 1e-4)   # observer velocity (units of c)


def run_velocity(args, synth, spec, cos, length, world, rank, local, dist):
    """The velocity-field build of the map driver (hmaps.cpp:360-455) on the
    benchmark octree: one step = one complete deposit of the particles
    (BEGIN, the particles, FINISH: Hmaps::CreateOctreeVelocityWithTSC at
    every level, normalisation, parent fill), particles resident on the
    device; e2e the same through mpf_velocity_deposit from host arrays.
    Beside it, the benchmark rays traced with the deposited field and an
    observer velocity (the Doppler redshift) against the same batches on the
    plain octree, and parity against the C oracle: a 65 536-particle deposit
    cell by cell and 48 rays with the Doppler term."""
    import torch
    torch.cuda.set_device(local)
    pkg = importlib.import_module(PKG)
    importlib.import_module(PKG + ".build").build()
    capi = importlib.import_module(PKG + ".capi")
    lib = pkg.library()
    rec = octree_records(synth, spec)
    tree = pkg.Octree.from_records(rec)
    info = tree.info
    cosmo = pkg.Cosmology(*cos)
    npart = args.particles
    pos, vel = synth.velocity_particles(rec, npart, seed=17)
    dev = torch.device("cuda", local)
    d_pos = torch.from_numpy(pos).to(dev)
    d_vel = torch.from_numpy(vel).to(dev)
    stream = torch.cuda.current_stream(dev)
    sh = stream.cuda_stream

    def deposit():
        tree.deposit_velocity_device(d_pos.data_ptr(), d_vel.data_ptr(), npart, "tsc", stream=sh)

    for _ in range(args.warmup):
        deposit()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            deposit()
        ev1.record(stream)
        torch.cuda.synchronize()
    dep_ms = ev0.elapsed_time(ev1) / args.steps
    value = npart / (dep_ms / 1000.0)
    pairs = tree.deposit_pairs()
    v_dev, rho_dev = tree.velocity()
    # end to end: host arrays through the public call
    e2e_t = []
    for _ in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tree.deposit_velocity(pos, vel, "tsc")
        e2e_t.append(time.perf_counter() - t0)
    v2, r2 = tree.velocity()
    deterministic = bool(np.array_equal(v2.view(np.uint32), v_dev.view(np.uint32)) and
                         np.array_equal(r2.view(np.uint32), rho_dev.view(np.uint32)))
    e2e_value = npart / (sum(e2e_t) / len(e2e_t))
    peak, peak_kind = measured_peak_hbm()
    # a scatter deposit's payload: every particle read (24 B), every contribution a
    # read-modify-write of its cell's mass and velocity (2 x 20 B)
    bytes_per_deposit = npart * 24 + pairs * 40
    achieved = bytes_per_deposit / (dep_ms / 1000.0) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": None, "peak_source": peak_kind,
                "bytes_per_deposit": {"particles_x_24": npart * 24, "pairs_x_40": pairs * 40},
                "note": "payload of a scatter deposit; the reference-order sort of the (cell, particle, vertex) "
                        "pairs (7 radix passes of 16 B per pair) is on top of it"}

    # the benchmark rays with the deposited field and an observer velocity, and on the plain octree
    launch = ray_grid()
    B = min(args.batch, launch.shape[0])
    d_launch = torch.from_numpy(launch).to(dev)
    d_steps = torch.zeros(B, dtype=torch.int64, device=dev)
    d_planes = torch.zeros(B * capi.MPF_PLANE_FIELDS, dtype=torch.float64, device=dev)
    d_status = torch.zeros(1, dtype=torch.int32, device=dev)
    planes = np.array([args.zstop])
    nb = launch.shape[0] // B

    def trace(vobs):
        p, keep = capi.make_params(length, nsteps=8, order=2, stop="redshift", planes=planes, jacobian=True,
                                   exact=False, vobs=vobs)
        total, ms = 0, 0.0
        for k in range(args.warmup + args.steps):
            off = (k % nb) * B
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            capi.check(lib.mpf_propagate_device(tree._h, cosmo._h, C.byref(p), B,
                                                C.c_void_p(d_launch.data_ptr() + off * 48),
                                                C.c_void_p(d_steps.data_ptr()), None, C.c_void_p(d_planes.data_ptr()),
                                                C.c_void_p(d_status.data_ptr()), C.c_void_p(sh)))
            e1.record(stream)
            torch.cuda.synchronize()
            if k >= args.warmup:
                ms += e0.elapsed_time(e1)
                total += int(d_steps.sum().item())
        return total / (ms / 1000.0)

    vel_rate = trace(VEL_VOBS)
    # parity: 48 rays with the Doppler term against the C oracle on the same field
    line_parity = {}
    cpu = None
    if rank == 0:
        import oracle as oracle_mod
        oracle_mod.build()
        acc = importlib.import_module(PKG + ".accuracy")
        O = oracle_mod.Oracle(rec, {"t": cos[0], "a": cos[1], "dadt": cos[2]}, length)
        O.fields[:, 0] = rho_dev
        O.set_velocity(v_dev, VEL_VOBS)
        rng = np.random.default_rng(5)
        sample = np.ascontiguousarray(launch[rng.choice(launch.shape[0], 48, replace=False)])
        s_r, f_r, p_r = O.propagate(sample, order=2, nsteps=8, stop="redshift", planes=planes, jacobian=True)
        s, f, pl, _ = pkg.propagate(tree, cosmo, sample, length, nsteps=8, order=2, stop="redshift", planes=planes,
                                    jacobian=True, exact=False, vobs=VEL_VOBS)
        rep = acc.compare(sample, s, f, pl, s_r, f_r, p_r)
        rep["within_tolerance"] = bool(acc.within(rep))
        line_parity["rays_with_doppler"] = rep
        # the deposit, cell by cell, on a 65 536-particle sample (the oracle on one thread: the CPU baseline)
        m = 65536
        t2 = pkg.Octree.from_records(rec)
        t2.deposit_velocity(pos[:m], vel[:m], "tsc")
        vg, rg = t2.velocity()
        t2.close()
        O2 = oracle_mod.Oracle(rec, {"t": cos[0], "a": cos[1], "dadt": cos[2]}, length)
        t0 = time.perf_counter()
        vo, ro = O2.deposit_velocity(pos[:m], vel[:m], "tsc")
        dt = time.perf_counter() - t0
        same = (vg.view(np.uint32) == vo.view(np.uint32)).all(1) & (rg.view(np.uint32) == ro.view(np.uint32))
        line_parity["deposit_sample"] = {"particles": m, "cells": int(rg.shape[0]),
                                         "cells_bit_identical": int(same.sum()), "all_identical": bool(same.all()),
                                         "against": "C oracle (bit-exact with the reference's -DVELOCITYFIELD build "
                                                    "on the fixtures)"}
        cpu = {"value": m / dt, "unit": VEL_UNIT, "cores": 1, "kind": "port",
               "sample": "%d particles, %.1f s, one thread (C oracle restating the reference's deposit in its "
                         "single-thread order)" % (m, dt)}
    tree.set_velocity(None)
    plain_rate = trace((0.0, 0.0, 0.0))
    config = {"workload": "velocity-field deposit of %d particles (cell-uniform positions, linear-flow velocities) "
                          "onto the AMR cone octree (256^3 base at level 10 refined to 14 in 2000 NFW haloes), TSC at "
                          "every level, then normalisation and parent fill" % npart,
              "particles": npart, "scheme": "TSC", "cells": int(info["cells"]),
              "levels": [info["level_min"], info["level_max"]], "pairs_per_deposit": pairs,
              "order": "particle then vertex per cell (the reference's single-thread order)",
              "l2": "octree larger than L2 (no flush)", "parallelism": "single GPU"}
    line = {"metric": VEL_METRIC, "value": value, "unit": VEL_UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dep_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config,
            "e2e": {"value": e2e_value, "unit": VEL_UNIT, "h2d_bytes_per_step": npart * 24, "d2h_bytes_per_step": 0},
            "gpu_launches": None, "roofline": roofline, "deterministic": deterministic,
            "trace": {"rays": "the benchmark's 1000x1000 grid in %d-ray batches, TSC, Jacobian at z=%g" % (B, args.zstop),
                      "vobs": list(VEL_VOBS), "velocity_field_photon_steps_per_s": vel_rate,
                      "plain_photon_steps_per_s": plain_rate, "ratio": vel_rate / plain_rate},
            "parity": line_parity, "clocks": clk.summary()}
    if cpu is not None:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
