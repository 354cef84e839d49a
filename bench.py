#!/usr/bin/env python3
"""Benchmark of CoMD's force-and-integrate step on GB300.

Metric: EAM atom-steps/s at 4M atoms on one GB300, mixed precision (FP32
pair terms, compensated per-atom sums, FP64 integration) against the plain
FP64 GPU kernel, with the force error of mixed vs FP64 stated.

Workload (the configuration the metric is quoted on): EAM Cu, Chebyshev
series (32 terms, fitted in FP64 on the GPU from the bundled Cu tables),
FCC 100x100x100 unit cells = 4,000,000 atoms, x-stretch (deformation
gradient) 1.05, box factor 1.5, seeded Maxwell-Boltzmann momenta at 300 K,
dt = 1 fs.  One step = one velocity-Verlet timestep of the reference's
nTimeSteps (advance positions dt/2, reBoxAll, force, advance momenta dt,
advance positions dt/2, reBoxAll).  Inputs are synthetic and seeded.

value: device-resident throughput, CUDA events over K graph replays.
e2e:   the same metric through the drop-in C ABI (comdgb_attach +
       comdgb_nTimeSteps(10) on a host simflat_t), host<->device copies of
       the whole simulation inside every call.
--impl reference: the reference's CPU path (oracle/_ref when it was built
from the reference sources on this machine, else the CPU oracle port)
with every host thread, each on an independent periodic sample.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOAD = {"name": "eam_cu_chebyshev_fcc100_stretch1.05_bf1.5_300K", "nx": 100, "ny": 100,
            "nz": 100, "defgrad": 1.05, "bf": 1.5, "temp_k": 300.0, "seed": 2026, "dt_s": 1e-15}
METRIC = "EAM atom-steps/s @4M atoms, 1 GB300: mixed vs FP64 at <=1e-5 force err"
UNIT = "atom-steps/s"
# algorithmic work (counted per unique in-cutoff pair / per atom; FMA = 2),
# the reference's Chebyshev arithmetic: its pass 1 sums three series (phi,
# phi', rho: 443 flops with r, dr and the sums) and its pass 3 one (rho': 132
# with the embedding force).  Here the density pass sums one series (rho)
# and the force pass three (phi, phi', rho'), so the counts swap kernels.
FLOPS_PASS1_PER_PAIR = 132    # density pass: rho by Clenshaw (+ r, dr, the sum)
FLOPS_PASS2_PER_PAIR = 443    # force pass: phi, phi', rho' by Clenshaw + the force
FLOPS_EMBED_PER_ATOM = 208    # F, F' per atom (fused into the density pass)
BYTES_VERLET_PER_ATOM = 120   # read r, p, f; write r, p (FP64)
BYTES_ADVPOS_PER_ATOM = 72    # read r, p; write r (FP64)
# CPU baselines (both arms): one process per host core, each an independent
# periodic sample of CPU_CELLS^3 FCC unit cells of the workload
CPU_CELLS = 30
CPU_COUNTING = ("atom-steps counted as the reference's own us/atom print counts them "
                "(src-flat/docompute.c:203-204): N * (n+1) force calls per nTimeSteps(n)")
# tolerances of the mixed path against the FP64 oracle (relative to the
# oracle's largest magnitude unless stated); tests/test_mixed_vs_oracle.py
# asserts the same values at 256,000 atoms
ORACLE_TOL = {"f_rel_rms": 1e-5, "f_max_rel": 1e-4, "e_atom_max_rel": 1e-6, "rho_max_rel": 1e-6,
              "fi_max_rel": 1e-5, "e_per_atom_abs": 1e-8, "stress_rel": 1e-5,
              "virial_max_rel": 1e-5}


def env_rank():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Dist:
    """Barrier / max over ranks (gloo on CPU) when launched with N > 1."""

    def __init__(self, world):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x):
        if not self.dist:
            return x
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", str(self.index)], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def make_host_sim(cg, w, nx=None, ny=None, nz=None, disp=None, amp=0.0):
    pot = cg.eam_potential("cu")
    s = cg.fcc(nx or w["nx"], ny or w["ny"], nz or w["nz"], pot.ptr.contents.lat, w["defgrad"],
               w["bf"], pot)
    cg.seed(s, w["seed"], disp if disp is not None else cg.DISP_NONE, amp, w["temp_k"],
            pot.ptr.contents.mass)
    return pot, s


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def committed_traffic():
    """per-launch DRAM bytes of the dominant kernel from the committed ncu summary"""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


# ------------------------------------------------------------------ CPU arms
def _cpu_worker(barrier, queue, cells, steps, w, prefer_reference, index):
    """One CPU sample in its own process (the reference keeps static state,
    so samples never share an address space).  stdout is silenced because
    the reference prints while it sets up."""
    devnull = os.open(os.devnull, os.O_WRONLY)
    os.dup2(devnull, 1)
    sys.path.insert(0, ROOT)
    import oracle
    ref = oracle.ref_lib(cheby=True) if prefer_reference else None
    if ref is not None:
        L = ref.lib
        potdir = os.path.join(ROOT, "comd_gb300", "pots").encode()
        rp = L.refh_eam_load(potdir, b"cu")
        s = L.refh_fcc(cells, cells, cells, 3.615, w["defgrad"], w["bf"], rp, 1)
        L.refh_seed_apply(s, w["seed"] + index, 0, 0.0, w["temp_k"], 63.55)
        L.refh_rebox(s)

        def run():
            L.refh_ntimesteps(steps, s, w["dt_s"])
        kind = "reference"
    else:
        O = oracle.Oracle()
        pot = O.eam(os.path.join(ROOT, "comd_gb300", "pots"), "cu")
        s = O.fcc(cells, cells, cells, pot.contents.lat, w["defgrad"], w["bf"], pot)
        s.contents.ch_pot = O.cheby(pot, 32)
        O.seed(s, w["seed"] + index, 0, 0.0, w["temp_k"], pot.contents.mass)
        O.rebox(s)

        def run():
            O.steps(s, steps, w["dt_s"], oracle.KIND_EAM_CHEBY)
        kind = "port"
    natoms = s.contents.ntot
    barrier.wait()
    t0 = time.perf_counter()
    run()
    queue.put((natoms, time.perf_counter() - t0, kind))


def cpu_sample(procs, cells, steps, w, prefer_reference):
    """`procs` independent periodic samples (cells^3 FCC unit cells with the
    workload's stretch, box factor and temperature), one spawned process per
    host core, each running nTimeSteps(steps) of the reference's CPU path
    concurrently.  Returns (atom-steps/s, kind, description); atom-steps are
    counted as the reference counts them: N * (steps + 1) force calls."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(procs)
    queue = ctx.Queue()
    ps = [ctx.Process(target=_cpu_worker, args=(barrier, queue, cells, steps, w,
                                                prefer_reference, i)) for i in range(procs)]
    for p in ps:
        p.start()
    res = [queue.get(timeout=1800) for _ in ps]
    for p in ps:
        p.join()
    natoms = res[0][0]
    wall = max(r[1] for r in res)
    kind = res[0][2]
    value = sum(r[0] for r in res) * (steps + 1) / wall
    # one core: the median process's own rate (the reference is serial)
    one_core = statistics.median(r[0] * (steps + 1) / r[1] for r in res)
    desc = (f"{procs} concurrent processes, each an independent periodic sample of {natoms} "
            f"atoms ({cells}^3 FCC cells, stretch {w['defgrad']}, box factor {w['bf']}, "
            f"{w['temp_k']} K momenta), nTimeSteps({steps}) of EAM Chebyshev FP64; "
            f"slowest sample {wall:.1f} s")
    return value, kind, desc, one_core


def cpu_threads():
    return max(1, min(os.cpu_count() or 1, 72))


def reference_arm(args):
    rank, world, _ = env_rank()
    if rank != 0:
        return 0
    threads = cpu_threads()
    w = WORKLOAD
    # each step: one nTimeSteps(1) per thread on an independent sample of
    # CPU_CELLS^3 cells (the GPU arm's cpu_baseline sample), about 3 s; only a
    # run of more than 60 steps shrinks it to stay within a few minutes
    total_steps = args.steps + args.warmup
    cells = CPU_CELLS
    if total_steps > 60:
        cells = max(8, int(CPU_CELLS * (60.0 / total_steps) ** (1 / 3)))
    for _ in range(args.warmup):
        cpu_sample(threads, cells, 1, w, True)
    vals, ones = [], []
    kind = desc = None
    for _ in range(args.steps):
        v, kind, desc, one = cpu_sample(threads, cells, 1, w, True)
        vals.append(v)
        ones.append(one)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded FCC Cu lattice, 300 K momenta)",
            "config": {"workload": w["name"], "atoms": 4_000_000, "potential": "EAM Cu Chebyshev",
                       "sample": desc},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": desc, "counting": CPU_COUNTING,
                             "one_core": {"value": statistics.median(ones), "unit": UNIT}},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm
def per_atom(s):
    """by-id copies of the force-call outputs of a host simflat_t"""
    from comd_gb300.abi import by_id
    f = by_id(s, "f")
    return {"f": f[:, :3].copy(), "e": f[:, 3].copy(), "rho": by_id(s, "rho").copy(),
            "fi": by_id(s, "fi").copy()}


def oracle_check(s, pot, mix, e_mix, st_mix, w_mix):
    """The FP64 oracle's force call and virial on the positions of host
    simflat_t s (one core), against the mixed-precision results: relative
    RMS and maximum errors of every output (eam.c:534-545, 586-594, 644-657)
    with the tolerances they are held to."""
    import oracle
    O = oracle.Oracle()
    t0 = time.perf_counter()
    so = O.clone(s)
    try:
        so.contents.ch_pot = O.cheby(pot.ptr, 32)
        if O.force(so, oracle.KIND_EAM_CHEBY):
            raise RuntimeError("oracle force call failed")
        orc = per_atom(so)
        w_orc, _, _ = O.virial(so, oracle.KIND_EAM_CHEBY)
        e_orc, st_orc = so.contents.e, so.contents.stress
    finally:
        O.free(so)
    n = len(orc["f"])

    def rms(a, b):
        return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))

    def mx(a, b):
        return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

    rec = {"f_rel_rms": rms(mix["f"], orc["f"]), "f_max_rel": mx(mix["f"], orc["f"]),
           "e_atom_rel_rms": rms(mix["e"], orc["e"]), "e_atom_max_rel": mx(mix["e"], orc["e"]),
           "rho_rel_rms": rms(mix["rho"], orc["rho"]), "rho_max_rel": mx(mix["rho"], orc["rho"]),
           "fi_rel_rms": rms(mix["fi"], orc["fi"]), "fi_max_rel": mx(mix["fi"], orc["fi"]),
           "e_per_atom_abs": abs(e_mix - e_orc) / n, "e_total_oracle_ha": e_orc,
           "stress_rel": abs(st_mix - st_orc) / abs(st_orc),
           "virial_max_rel": mx(w_mix, w_orc), "virial_oracle_ha": [float(x) for x in w_orc]}
    rec["within_tolerance"] = all(rec[k] <= v for k, v in ORACLE_TOL.items())
    rec["tolerances"] = ORACLE_TOL
    rec["atoms"] = n
    rec["oracle_seconds"] = time.perf_counter() - t0
    return rec


def gpu_arm(args):
    import comd_gb300 as cg

    rank, world, local = env_rank()
    dist = Dist(world)
    dev = local
    w = WORKLOAD
    cg.load()
    pot, s = make_host_sim(cg, w)
    rc = cg.load().comdgb_rebox_host(s, 1, dev)  # initSimFromCmdLine's reBoxAll
    if rc:
        raise cg.ComdgbError(rc, cg.lib.last_error())
    natoms = s.contents.ntot
    dt = w["dt_s"]

    mixed = cg.DeviceSim(s, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED, device=dev,
                                    cheby_from_host=False))
    h0_e, _ = mixed.force()
    h0 = h0_e + mixed.kinetic()
    mixed.steps(args.warmup, dt)
    mixed.synchronize()

    persistent, skin, builds0 = mixed.list_info()
    clocks = ClockSampler(dev)
    clocks.start()
    dist.barrier()
    mixed.synchronize()
    step_ms, span_ms, kern_ms = mixed.timed_steps(args.steps, dt)
    mixed.synchronize()
    dist.barrier()
    clk = clocks.stop()
    lists = {"persistent": persistent, "skin_A": skin,
             "builds_in_timed_steps": mixed.list_info()[2] - builds0}
    elapsed_s = dist.max(span_ms / 1e3)
    value = dist.sum(natoms * args.steps) / elapsed_s
    pairs = mixed.pair_count()
    # before any recapture below: the step graphs' kernels, plus the
    # conditional rebuild section's once per rebuild
    launches = (mixed.step_launches(args.steps)
                + lists["builds_in_timed_steps"] * mixed.rebuild_launches())

    # energy drift over 1000 steps (warmup + timed + the rest, untimed)
    done = args.warmup + args.steps
    drift = None
    if args.drift_steps > done:
        mixed.steps(args.drift_steps - done, dt)
        e1, _ = mixed.force()
        drift = abs(e1 + mixed.kinetic() - h0) / natoms

    # accuracy on the same (thermalised) state: the mixed force call and
    # virial, the plain FP64 GPU kernel, and the FP64 oracle (the reference's
    # double-precision force call restated on the CPU)
    e_mix, st_mix = mixed.force()
    w_mix, _, _ = mixed.virial()
    mixed.download(s)
    mix = per_atom(s)
    fp64_value = fp64_ms = None
    ferr = None
    if not args.no_fp64:
        fp64 = cg.DeviceSim(s, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, device=dev,
                                       cheby_from_host=False))
        fp64.force()
        fp64.download(s)
        f64 = per_atom(s)["f"]
        ferr = float(np.sqrt(np.mean((mix["f"] - f64) ** 2)) / np.sqrt(np.mean(f64 ** 2)))
        fp64.steps(1, dt)
        fp64.synchronize()
        st64, span64, _ = fp64.timed_steps(args.fp64_steps, dt)
        fp64_ms = span64 / args.fp64_steps
        fp64_value = natoms / (fp64_ms / 1e3)
        fp64.close()
    vs_oracle = None
    if rank == 0 and not args.no_oracle:
        vs_oracle = oracle_check(s, pot, mix, e_mix, st_mix, w_mix)

    # mixed precision with the reference's series evaluated in FP32 for every
    # pair (no segment table): the same algorithm as the FP64 kernel, so
    # against it the speed-up of precision alone
    series_ms = None
    if args.series_steps > 0:
        mixed.set_pair_table(False)
        mixed.steps(2, dt)
        mixed.synchronize()
        _, span_s, _ = mixed.timed_steps(args.series_steps, dt)
        series_ms = span_s / args.series_steps
        mixed.set_pair_table(True)

    # e2e through the drop-in C ABI on the host simflat_t
    e2e = None
    if not args.no_e2e:
        import ctypes as C
        L = cg.load()
        o = cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED, device=dev, cheby_from_host=False)
        cg.lib.check(L.comdgb_attach(s, C.byref(o)))
        calls, per_call = args.e2e_calls, 10
        L.comdgb_nTimeSteps(per_call, s, dt)  # warm-up: graph capture, pinning
        b0 = (C.c_longlong(), C.c_longlong())
        cg.lib.check(L.comdgb_transfer_bytes(s, C.byref(b0[0]), C.byref(b0[1])))
        dist.barrier()
        import gc
        gc.collect()
        gc.disable()  # no collector pause inside the host-timed loop
        t0 = time.perf_counter()
        call_ms = []
        for _ in range(calls):
            tc = time.perf_counter()
            e = L.comdgb_nTimeSteps(per_call, s, dt)
            call_ms.append((time.perf_counter() - tc) * 1e3)
            if e != e:
                raise cg.ComdgbError(-30, cg.lib.last_error())
        t1 = time.perf_counter()
        gc.enable()
        dist.barrier()
        e2e_s = dist.max(t1 - t0)
        b1 = (C.c_longlong(), C.c_longlong())
        cg.lib.check(L.comdgb_transfer_bytes(s, C.byref(b1[0]), C.byref(b1[1])))
        L.comdgb_detach(s)
        # bytes the library copied in the timed calls (each box's slots up to
        # the largest occupancy; the upload carries the state, the download
        # the state and the forces)
        h2d = (b1[0].value - b0[0].value) // calls
        d2h = (b1[1].value - b0[1].value) // calls
        e2e = {"value": dist.sum(natoms * calls * per_call) / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": h2d // per_call, "d2h_bytes_per_step": d2h // per_call,
               "call": f"comdgb_nTimeSteps({per_call}) on a host simflat_t (pinned), "
                       "full state copied up and back every call",
               "call_ms": [round(x, 2) for x in call_ms]}

    # roofline of the dominant kernel group
    peaks = measured_peaks()
    fp32_peak = cg.lib.fp32_peak_tflops(dev)
    dom = max(kern_ms, key=kern_ms.get)
    groups = {}
    for name, ms in kern_ms.items():
        g = {"ms": ms, "share": ms / sum(kern_ms.values())}
        if name == "force_pass1":
            fl = FLOPS_PASS1_PER_PAIR * pairs + FLOPS_EMBED_PER_ATOM * natoms
            g.update(bound="fp32", achieved=fl / (ms / 1e3) / 1e12, unit="TFLOP/s")
        elif name.startswith("force_pass2"):  # (force order: with the step's update)
            fl = FLOPS_PASS2_PER_PAIR * pairs
            g.update(bound="fp32", achieved=fl / (ms / 1e3) / 1e12, unit="TFLOP/s")
        elif name.startswith("advance_velocity"):
            g.update(bound="hbm", achieved=BYTES_VERLET_PER_ATOM * natoms / (ms / 1e3) / 1e9,
                     unit="GB/s")
        elif name.startswith("advance_positions"):
            g.update(bound="hbm", achieved=BYTES_ADVPOS_PER_ATOM * natoms / (ms / 1e3) / 1e9,
                     unit="GB/s")
        if "bound" in g:
            pk = fp32_peak if g["bound"] == "fp32" else peaks.get("hbm_gbs", 6800.0)
            g["peak"] = pk
            g["frac"] = g["achieved"] / pk
        groups[name] = g
    dg = groups[dom]
    traffic = committed_traffic().get(dom)
    limits = committed_traffic().get("limits", {})
    roofline = {"kernel": dom, "bound": dg.get("bound"), "achieved": dg.get("achieved"),
                "peak": dg.get("peak"), "unit": dg.get("unit"), "frac": dg.get("frac"),
                "traffic": traffic,
                # the unit the kernel is really bound by, from the committed ncu capture
                "measured_limit": limits.get(dom),
                "peak_source": ("FP32 FMA throughput measured on this GPU by "
                                "comdgb_fp32_fma_peak (no FP32 figure in MEASURED_PEAKS.json)"
                                if dg.get("bound") == "fp32" else "MEASURED_PEAKS.json hbm_gbs"),
                "algorithmic": (f"{FLOPS_PASS2_PER_PAIR} flops/unique pair, {pairs} pairs"
                                if dom.startswith("force_pass2") else
                                f"{FLOPS_PASS1_PER_PAIR} flops/unique pair + "
                                f"{FLOPS_EMBED_PER_ATOM}/atom, {pairs} pairs")}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, kind, desc, one = cpu_sample(cpu_threads(), args.cpu_cells, 1, w, True)
        cpu = {"value": v, "unit": UNIT, "cores": cpu_threads(), "kind": kind, "sample": desc,
               "counting": CPU_COUNTING,
               # the serial reference on one core (the median process's own rate)
               "one_core": {"value": one, "unit": UNIT}}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_s * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded FCC Cu lattice, 300 K momenta)",
        "config": {"workload": w["name"], "atoms": natoms, "potential": "EAM Cu Chebyshev 32",
                   "precision": "mixed (FP32 pairs, Kahan FP32 sums, FP64 integration)",
                   "boxes": s.contents.nboxes, "nbx": list(s.contents.nbx),
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (~1.1 GB device state per step)",
                   "dt_fs": 1.0},
        "fp64_gpu": {"value": fp64_value, "ms_per_step": fp64_ms, "steps": args.fp64_steps},
        "mixed_vs_fp64": (value / world / fp64_value) if fp64_value else None,
        "mixed_series_gpu": {"ms_per_step": series_ms, "steps": args.series_steps,
                             "value": natoms / (series_ms / 1e3) if series_ms else None,
                             "what": "mixed precision, the 32-term series in FP32 for every "
                                     "pair (segment table off)"},
        "speedup_split": {
            "precision_only": (fp64_ms / series_ms) if fp64_ms and series_ms else None,
            "algorithm_only": (series_ms / (elapsed_s * 1e3 / args.steps))
                              if series_ms else None,
            "what": "precision_only = FP64 kernel / mixed with the series (both sum the "
                    "series per pair); algorithm_only = mixed with the series / mixed with "
                    "the segment table; their product is mixed_vs_fp64"},
        "force_rel_rms_mixed_vs_fp64": ferr,
        "force_rel_rms_mixed_vs_oracle": vs_oracle["f_rel_rms"] if vs_oracle else None,
        "accuracy_vs_oracle": vs_oracle,
        "energy_drift_ha_per_atom": drift, "drift_steps": args.drift_steps,
        "neighbour_lists": lists, "pairs_per_step": pairs, "pair_evals_per_s": pairs * args.steps / (span_ms / 1e3),
        "kernel_groups": groups, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "clocks": clk,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    mixed.close()
    cg.free_host(s)
    dist.close()
    return 0


# ------------------------------------------------------------ C4: batches
BATCH = {"replicas": 64, "edge": (8, 24), "temp_k": (100.0, 1200.0), "seed": 4242, "steps": 50,
         "bf": (1.0, 1.2, 1.4), "skin": (0.3, 0.4, 0.5, 0.6)}


def batch_arm(args):
    """64 EAM Cu Chebyshev replicas (mixed precision) of seeded uneven size,
    edge U{8..24} unit cells, temperature U(100, 1200) K, advanced together:
    a 50-step loop captured as one CUDA graph over all replicas.  The box
    factor and the skin, then the launch shapes (the list build's threads per
    box and atoms per candidate load, the force pass's threads per CTA), are
    chosen by the library's autotuner (comdgb_batch_autotune, timing every
    candidate on the batch itself, cached per GPU and system); the result is
    set against the same 64 systems run one after another with the same
    settings.  The launch structure is measured too: the cost of one kernel
    node of the step graph against one grid-wide barrier of a persistent
    kernel (comdgb_graph_node_cost, comdgb_grid_barrier_cost)."""
    import comd_gb300 as cg
    rng = np.random.default_rng(BATCH["seed"])
    R = BATCH["replicas"]
    edges = rng.integers(BATCH["edge"][0], BATCH["edge"][1] + 1, R)
    temps = rng.uniform(BATCH["temp_k"][0], BATCH["temp_k"][1], R)
    pot = cg.eam_potential("cu")
    lat, mass = pot.ptr.contents.lat, pot.ptr.contents.mass
    natoms = int(sum(4 * int(n) ** 3 for n in edges))
    nsteps = BATCH["steps"]

    def build(bf):
        sims = []
        for r in range(R):
            n = int(edges[r])
            s = cg.fcc(n, n, n, lat, 1.0, bf, pot)
            cg.seed(s, BATCH["seed"] + r, cg.DISP_NONE, 0.0, float(temps[r]), mass)
            sims.append(s)
        return sims

    def free(sims):
        for s in sims:
            cg.free_host(s)

    def o(skin):
        return cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED, skin=skin)

    base = build(1.0)
    try:
        t0 = time.perf_counter()
        tune = cg.batch_autotune(base, o(None), BATCH["bf"], BATCH["skin"], steps=20,
                                 cache_path=args.tune_cache or None)
        tune_s = time.perf_counter() - t0
    finally:
        free(base)
    sims = build(tune.box_factor)
    try:
        b = cg.Batch(sims, o(tune.skin))
        try:
            b.apply_tune(tune)
            b.graph_steps(nsteps)  # capture + warm
            clk = ClockSampler(0)
            clk.start()
            times = [b.graph_steps(nsteps) for _ in range(max(args.steps // nsteps, 3))]
            clocks = clk.stop()
            e, _ = b.energies()
            b.steps(2)  # the step graphs (their kernel counts), after the timed loops
            per_step = b.step_launches(nsteps) / nsteps
        finally:
            b.close()
        t_batch = statistics.median(times)
        # the same systems one after another
        t_seq = 0.0
        for r in range(R):
            d = cg.DeviceSim(sims[r], o(tune.skin))
            try:
                if d.list_info()[0]:
                    d.apply_tune(tune)
                d.graph_steps(nsteps)
                t_seq += d.graph_steps(nsteps)
            finally:
                d.close()
    finally:
        free(sims)
    node_us, barrier_us = cg.lib.launch_probes(0)
    value = natoms * nsteps / (t_batch * 1e-3)
    seq = natoms * nsteps / (t_seq * 1e-3)
    ms_step = t_batch / nsteps
    print(json.dumps({
        "metric": "EAM atom-steps/s, 64 uneven replicas in one launch per kernel, 1 GB300",
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": nsteps, "higher_is_better": True,
        "dtype": "f32+f64", "data": "synthetic (seeded FCC Cu replicas)",
        "config": {"workload": "eam_cu_chebyshev_64_replicas_edge8-24_100-1200K",
                   "replicas": R, "atoms": natoms, "edges_min_max": [int(edges.min()),
                                                                    int(edges.max())],
                   "loop": f"{nsteps} steps captured as one CUDA graph"},
        "ms_per_loop": t_batch, "sequential_64": {"value": seq, "ms_total": t_seq},
        "speedup_vs_sequential": value / seq,
        "autotune": {"chosen": tune.as_dict(), "seconds": tune_s,
                     "candidates": {"box_factor": BATCH["bf"], "skin_A": BATCH["skin"],
                                    "build_threads": [64, 128, 256], "build_atoms": [2, 4, 8],
                                    "pass2_threads": [128, 256, 512]},
                     "cache": args.tune_cache or None},
        "launch_structure": {
            "kernels_per_step_graph": per_step, "graph_node_us": node_us,
            "grid_barrier_us": barrier_us, "ms_per_step": ms_step,
            "node_overhead_frac": per_step * node_us * 1e-3 / ms_step,
            "what": "a persistent step kernel would save at most the graph's kernel nodes "
                    "(kernels_per_step_graph x graph_node_us) and pay a grid-wide barrier "
                    "per phase instead"},
        "energy_per_atom_ha": {"min": float(min(e / (4 * edges ** 3))),
                               "max": float(max(e / (4 * edges ** 3)))},
        "clocks": clocks}))
    return 0


# ---------------------------------------------------------- C5: adjoint
def adjoint_arm(args):
    """Gradients on 10 seeded FCC 40^3 EAM Cu configurations (256,000 atoms,
    Gaussian displacements sigma 0.05*sqrt(T/300 K) A and momenta at
    300/600/900 K): force-matching loss against forces of +-2 % seeded
    perturbed Chebyshev coefficients, its gradient in the 96 coefficients
    (timed), central differences (h = 1e-6 relative) on config 0, LJ
    epsilon/sigma gradients on config 0's lattice, and the energy gradient
    through 200 velocity-Verlet steps (checkpoints every 20) on a 20^3 lattice
    against central differences of whole trajectories."""
    import comd_gb300 as cg
    from comd_gb300.abi import by_id
    pot = cg.eam_potential("cu")
    lat, mass = pot.ptr.contents.lat, pot.ptr.contents.mass
    rng = np.random.default_rng(515)
    temps = [300.0, 600.0, 900.0]
    rows = []
    fd_report = {}

    def lattice(n, temp, seed, p=pot, m=mass):
        s = cg.fcc(n, n, n, lat, 1.0, 1.0, p)
        cg.seed(s, seed, cg.DISP_GAUSSIAN, 0.05 * (temp / 300.0) ** 0.5, temp, m)
        return s

    for k in range(10):
        temp = temps[k % 3]
        s = lattice(40, temp, 700 + k)
        d = cg.DeviceSim(s, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64))
        try:
            c, x0, xn = d.get_cheby()
            d.set_cheby(c * (1 + 0.02 * rng.uniform(-1, 1, c.size)), x0, xn)
            d.force()
            d.download(s)
            target = by_id(s, "f")[:, :3].copy()
            d.set_cheby(c, x0, xn)
            d.force_loss_grad(target)  # warm
            t0 = time.perf_counter()
            loss, g = d.force_loss_grad(target)
            t_grad = time.perf_counter() - t0
            rows.append({"temp_k": temp, "loss": loss, "grad_norm": float(np.linalg.norm(g)),
                         "grad_ms": t_grad * 1e3})
            if k == 0:
                errs = []
                for q in range(3):
                    j = int(np.argmax(np.abs(g[32 * q:32 * q + 32]))) + 32 * q
                    for jj in (j, 32 * q + 7):
                        h = 1e-6 * max(abs(c[jj]), 1e-3 * np.abs(c[32 * q:32 * q + 32]).max())
                        v = []
                        for sg in (1, -1):
                            cc = c.copy()
                            cc[jj] += sg * h
                            d.set_cheby(cc, x0, xn)
                            v.append(d.force_loss_grad(target)[0])
                        fd = (v[0] - v[1]) / (2 * h)
                        errs.append(abs(g[jj] - fd) / max(abs(fd), 1e-3 * np.abs(g).max()))
                d.set_cheby(c, x0, xn)
                fd_report["eam_force_loss_fd_max_rel_err"] = float(max(errs))
                fd_report["eam_force_loss_fd_components"] = len(errs)
        finally:
            d.close()
            if k:
                cg.free_host(s)
            else:
                s0 = s
    # LJ epsilon / sigma on configuration 0's lattice (the default LJ run's parameters)
    ev = cg.lib.EV_TO_HA
    sig, eps = 2.315, 0.167 * ev
    ljp = cg.lj_potential(sig, eps, 2.5 * sig, 63.55)
    sl = cg.fcc(40, 40, 40, lat, 1.0, 1.0, ljp)
    cg.seed(sl, 700, cg.DISP_GAUSSIAN, 0.05, 300.0, 63.55)
    d = cg.DeviceSim(sl, cg.opts(cg.POT_LJ, cg.PREC_FP64))
    try:
        d.set_lj(eps * 1.02, sig * 0.99)
        d.force()
        d.download(sl)
        tl = by_id(sl, "f")[:, :3].copy()
        d.set_lj(eps, sig)
        U, gu = d.energy_grad()
        L, gl = d.force_loss_grad(tl)
        errs = []
        for i, (de, ds) in enumerate([(1, 0), (0, 1)]):
            h = 1e-6 * (eps if de else sig)
            v = []
            for sg in (1, -1):
                d.set_lj(eps + sg * de * h, sig + sg * ds * h)
                v.append(d.force_loss_grad(tl)[0])
            errs.append(abs(gl[i] - (v[0] - v[1]) / (2 * h)) / abs(gl[i]))
        fd_report["lj_force_loss_fd_max_rel_err"] = float(max(errs))
        fd_report["lj_grad_energy"] = [float(x) for x in gu]
        fd_report["lj_grad_loss"] = [float(x) for x in gl]
    finally:
        d.close()
        cg.free_host(sl)
        cg.free_host(s0)
    # trajectory adjoint: timed on 20^3 (32,000 atoms); checked against whole-
    # trajectory differences on 6^3 at 300 K, where few pairs cross the cutoff
    st = lattice(20, 600.0, 900)
    d = cg.DeviceSim(st, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, per_step_lists=True))
    try:
        t0 = time.perf_counter()
        J, g = d.traj_energy_grad(200, 1e-15, 20)
        t_traj = time.perf_counter() - t0
        natoms_t = st.contents.ntot
    finally:
        d.close()
        cg.free_host(st)
    st = lattice(6, 300.0, 901)
    d = cg.DeviceSim(st, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_FP64, per_step_lists=True))
    try:
        c, x0, xn = d.get_cheby()
        Jc, g = d.traj_energy_grad(200, 1e-15, 20)
        errs, skipped = [], 0
        cand = [int(np.argmax(np.abs(g[32 * q:32 * q + 32]))) + 32 * q for q in range(3)]
        for jj in cand + [1, 5, 8, 33, 40, 66, 70]:
            q = jj // 32
            h = 1e-6 * max(abs(c[jj]), 1e-3 * np.abs(c[32 * q:32 * q + 32]).max())
            fds = []
            for hh in (h, h / 4):
                v = []
                for sg in (1, -1):
                    cc = c.copy()
                    cc[jj] += sg * hh
                    d.set_cheby(cc, x0, xn)
                    d.upload(st)
                    v.append(d.steps(200)[0])
                fds.append((v[0] - v[1]) / (2 * hh))
            scale = max(abs(fds[0]), 1e-3 * np.abs(g).max())
            if abs(fds[0] - fds[1]) > 1e-6 * scale:
                skipped += 1  # a cutoff crossing inside the difference bracket
                continue
            errs.append(abs(g[jj] - fds[0]) / scale)
        fd_report["trajectory"] = {"atoms": natoms_t, "steps": 200, "every": 20,
                                   "J_ha": J, "seconds": t_traj,
                                   "fd_check_atoms": st.contents.ntot,
                                   "fd_max_rel_err": float(max(errs)) if errs else None,
                                   "fd_components": len(errs), "fd_skipped_crossing": skipped}
    finally:
        d.close()
        cg.free_host(st)
    print(json.dumps({
        "metric": "adjoint: force-matching gradient (96 Chebyshev coefficients) per 256k-atom "
                  "EAM Cu configuration, FP64, 1 GB300",
        "value": statistics.median(r["grad_ms"] for r in rows), "unit": "ms",
        "higher_is_better": False, "dtype": "f64", "data": "synthetic (seeded FCC Cu)",
        "config": {"workload": "eam_cu_chebyshev_fcc40_x10_300-900K_adjoint"},
        "configs": rows, "checks": fd_report}))
    return 0


def analysis_arm(args):
    """The analyses beside the step, on the bundled 262,144-atom Ag structure
    (the reference's data/262k.inp.gz, EAM Ag Chebyshev, box factor 1):
    reading the clsman file (host parse + device binning), the virial tensor
    (force call + virial pass, mixed precision), the centrosymmetry
    parameter (exact pairing minimum and the greedy variant), the id-order
    gather and the three clsman writers.  Each op is timed as its C ABI call
    (wall clock, the call synchronises), median of K calls after one warm-up.
    CPU baseline: the oracle's restatements of the virial and the exact
    centrosymmetry on the 8,192-atom Ag file, one core."""
    import gzip
    import tempfile
    import comd_gb300 as cg
    pot = cg.eam_potential("ag")
    path = os.path.join(cg.DATA_DIR, "262k.inp.gz")
    k = max(3, min(args.steps, 10))
    ops = {}

    def timed(name, fn, atoms):
        fn()
        ts = []
        for _ in range(k):
            t0 = time.perf_counter()
            fn()
            ts.append(time.perf_counter() - t0)
        ms = statistics.median(ts) * 1e3
        ops[name] = {"ms": ms, "atoms_per_s": atoms / (ms * 1e-3)}

    sims = []

    def read():
        s = cg.read_clsman(path, pot, 1.0, 0)
        sims.append(s)
    timed("read_clsman_gz_device_binning", read, 262144)
    s = sims.pop()
    for q in sims:
        cg.free_host(q)
    assert cg.load().comdgb_rebox_host(s, 1, 0) == 0
    n = s.contents.ntot
    d = cg.DeviceSim(s, cg.opts(cg.POT_EAM_CHEBY, cg.PREC_MIXED))
    tmp = tempfile.mkdtemp(prefix="comdgb_")
    try:
        timed("force_mixed", lambda: d.force(), n)
        timed("virial_mixed", lambda: d.virial(), n)
        timed("centrosymmetry_exact", lambda: d.centrosymmetry(), n)
        timed("centrosymmetry_greedy", lambda: d.centrosymmetry(0, True), n)
        timed("gather_by_id", lambda: d.gather(), n)
        timed("write_binary", lambda: d.write_clsman(os.path.join(tmp, "a.bin")), n)
        timed("write_text_gz", lambda: d.write_clsman(os.path.join(tmp, "a.txt.gz"),
                                                      cg.CLSMAN_TEXT_GZ, "bench\n"), n)
        timed("write_text", lambda: d.write_clsman(os.path.join(tmp, "a.txt"),
                                                   cg.CLSMAN_TEXT, "bench\n"), n)
        for f in ("a.bin", "a.txt.gz", "a.txt"):
            ops["write_" + f.replace(".", "_") + "_bytes"] = os.path.getsize(os.path.join(tmp, f))
            os.remove(os.path.join(tmp, f))
    finally:
        d.close()
        cg.free_host(s)
        os.rmdir(tmp)
    cpu = None
    if not args.no_cpu:
        import oracle
        O = oracle.Oracle()
        with tempfile.NamedTemporaryFile(suffix=".inp") as f:
            f.write(gzip.open(os.path.join(cg.DATA_DIR, "8k.inp.gz")).read())
            f.flush()
            op = O.eam(os.path.join(ROOT, "comd_gb300", "pots"), "ag")
            so = O.read_clsman(f.name, op, 1.0)
        so.contents.ch_pot = O.cheby(op, 32)
        O.rebox(so)
        O.force(so, oracle.KIND_EAM_CHEBY)
        t0 = time.perf_counter()
        O.virial(so, oracle.KIND_EAM_CHEBY, atoms=True)
        t_vir = time.perf_counter() - t0
        t0 = time.perf_counter()
        O.centro(so)
        t_cen = time.perf_counter() - t0
        na = so.contents.ntot
        O.free(so)
        cpu = {"value": na / t_cen, "unit": "atoms/s", "cores": 1, "kind": "port",
               "sample": f"oracle centrosymmetry (exact) of the {na}-atom Ag file, {t_cen:.2f} s",
               "virial_atoms_per_s": na / t_vir}
    line = {"metric": "analysis: centrosymmetry (exact) throughput, 262,144-atom Ag structure, "
                      "1 GB300",
            "value": ops["centrosymmetry_exact"]["atoms_per_s"], "unit": "atoms/s",
            "higher_is_better": True, "dtype": "f64", "data": "bundled Ag structure (262k)",
            "config": {"workload": "ag262k_clsman_analysis"}, "ops": ops, "cpu_baseline": cpu,
            "vs_baseline": None}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=20)
    ap.add_argument("--series-steps", type=int, default=20,
                    help="steps of the mixed-precision run with the series evaluator")
    ap.add_argument("--tune-cache", default="",
                    help="autotune cache file of the batch workload (default: none)")
    ap.add_argument("--no-oracle", action="store_true",
                    help="skip the FP64 oracle force call on the full-size state")
    ap.add_argument("--drift-steps", type=int, default=1000)
    ap.add_argument("--e2e-calls", type=int, default=20)
    ap.add_argument("--cpu-cells", type=int, default=CPU_CELLS)
    ap.add_argument("--cells", type=int, default=0,
                    help="override the lattice to N^3 unit cells (profiling captures only)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="step",
                    choices=["step", "batch", "adjoint", "analysis"],
                    help="step: the headline 4M-atom step; batch: 64 replicas (C4); "
                         "adjoint: gradients (C5); analysis: virial, centrosymmetry and "
                         "clsman IO on the 262k Ag structure")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.cells:
        WORKLOAD.update(nx=args.cells, ny=args.cells, nz=args.cells,
                        name=WORKLOAD["name"].replace("fcc100", f"fcc{args.cells}"))
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "batch":
        return batch_arm(args)
    if args.workload == "adjoint":
        return adjoint_arm(args)
    if args.workload == "analysis":
        return analysis_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
