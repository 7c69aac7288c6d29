"""Benchmark of the superblock matvec (model_wave) on one or more GB300s.

Workload: the mid-chain superblock of the Hofstadter-Hubbard cylinder W=4,
L=32, phi=1/4 (Landau gauge), t=1, U=8, N_e=112 (1/8 hole doping), m=2000
kept multiplets per block -- the configuration the headline metric is quoted
on.  Block operators are seeded synthetic N(0,1) data with the sector
structure of such a step (see hofstadter_hubbard_tsc_gb300/synth.py); the term
list, 6j coefficients and task structure are the real ones.

One step = one H psi.  ``value`` is matvecs/s with psi and the operators
resident in HBM (CUDA events on the library's stream, L2 flushed between
steps); ``e2e`` is the same through the C-ABI call with host buffers
(hh_matvec_host: pinned H2D copy of psi, matvec, D2H copy of H psi every
step).  --impl reference times the CPU restatement of the reference's
model_wave (numpy, all host cores) on the same workload.

Sweep time, the metric's second half, is measured twice: on the 2x16 ladder
of the plain method (one whole finite sweep per arm at m = 256 and 512), and
as a window of mid-chain steps of the 4x32 cylinder at m = 2000 (the headline
configuration): the state is grown once by the infinite-system warm-up in
split precision (untimed), then the FP64 arm and the split-precision arm each
run the same K steps of the left-to-right sweep from one in-memory copy of it.
Multi-GPU: replicas only (the step does not exchange data): each rank runs the
workload, value = sum of matvecs over ranks / max time over ranks.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "matvecs/s & sweep time at fixed m, mixed+learned vs FP64 GPU, |dE/E|<=1e-8"
UNIT = "matvecs/s"


def _prec_codes():
    from hofstadter_hubbard_tsc_gb300 import _lib
    return {"fp64": _lib.HH_PREC_FP64, "bf16x6": _lib.HH_PREC_BF16X6, "bf16x3": _lib.HH_PREC_BF16X3}


PREC = _prec_codes()


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--precision", default="bf16x3", choices=["fp64", "bf16x6", "bf16x3"],
                   help="bf16x3: two BF16 parts, three products per real product; bf16x6: three parts, six")
    p.add_argument("--config", default="c2", choices=["c2", "c3", "c4", "c5"],
                   help="matvec workload: c2 Hubbard 4x32 phi=1/4 N_e=112 m=2000 (headline); c3 t-J 4x48 "
                        "J=0.4 phi=1/6 N_e=176 m=4000; c4 Hubbard 6x24 phi=1/3 N_e=132 m=6000 (mid-chain "
                        "superblocks, synthetic operators); c5 the synthetic block-sparse matvec (300 lognormal "
                        "sectors, median 96, max 2048, 12 terms, 8 uneven psi in one launch); --W/--L/--ne/--m "
                        "override c2's sizes")
    p.add_argument("--m", "--kept", dest="m", type=int, default=2000,
                   help="kept multiplets of the c2 workload (--kept under torchrun, whose own options "
                        "shadow --m)")
    p.add_argument("--W", type=int, default=4)
    p.add_argument("--L", type=int, default=32)
    p.add_argument("--ne", type=int, default=112)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-sample", type=int, default=1, help="matvecs in the CPU baseline sample")
    p.add_argument("--no-sweep", action="store_true", help="skip the sweep-time measurement")
    p.add_argument("--sweep-m", type=int, nargs="+", default=[256, 512],
                   help="kept multiplets of the sweep measurements (one timed finite sweep per precision)")
    p.add_argument("--sweep-precision", default="bf16x6", choices=["bf16x6", "bf16x3"],
                   help="split precision of the sweep's mixed arm (at m = 256-512 the matvecs are launch bound: "
                        "BF16x6 costs about the same as BF16x3 and keeps |dE/E| near 1e-10 instead of 1e-9)")
    p.add_argument("--no-energy-check", action="store_true",
                   help="skip the Lanczos (100 vectors) in FP64 and in split precision from one start vector "
                        "on the matvec workload (|dE/E|, outside the timed region)")
    p.add_argument("--no-window", action="store_true",
                   help="skip the sweep window of the 4x32 cylinder at m = 2000")
    p.add_argument("--window-m", type=int, default=2000, help="kept multiplets of the sweep window")
    p.add_argument("--window-steps", type=int, default=4, help="timed mid-chain steps per arm in the sweep window")
    p.add_argument("--window-L", type=int, default=32, help="cylinder length of the sweep window (N_e = 3.5 L)")
    p.add_argument("--no-configs", action="store_true",
                   help="skip the c3 / c4 matvec measurements reported beside the headline line")
    p.add_argument("--eigensolver", default="own", choices=["own", "cusolver"],
                   help="density-matrix eigensolver of both arms: the library's own FP64 kernels (default) or "
                        "cuSOLVER zheevd above 32 states (comparison)")
    return p.parse_args()


def max_over_ranks(x, dist, device):
    """The largest value of x over the ranks (x itself without a process
    group): the job's time is its slowest replica's."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(world_size, steps, t_max):
    """Whole-job throughput of independent replicas: every rank did `steps`
    matvecs in at most t_max seconds."""
    return world_size * steps / t_max


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
        return dist, rank, ws, local
    return None, rank, ws, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu):
        self.gpu, self.samples, self.proc = gpu, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=2)
        except Exception:
            self.proc.kill()
        sm = [float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for n, v in zip(names, s[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "_fallback": True}


def captured_traffic(workload, precision):
    """DRAM bytes per launch of the dominant (stage-2) kernel from the committed
    ncu capture of the same workload and precision (dram__bytes_read.sum +
    dram__bytes_write.sum), else None."""
    try:
        with open(os.path.join(ROOT, "profiles", "tc_stage2_traffic.json")) as f:
            t = json.load(f)
        if t.get("workload") == workload and t.get("precision") == precision:
            return float(t["dram_bytes_per_launch"])
    except Exception:
        pass
    return None


def fp64_peak_tflops():
    """Dense FP64 rate of this GPU, measured with cuBLAS DGEMM (torch.matmul, best of 5)."""
    try:
        import torch
        n = 4096
        a = torch.randn(n, n, dtype=torch.float64, device="cuda")
        b = torch.randn(n, n, dtype=torch.float64, device="cuda")
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e9
        for _ in range(5):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            torch.matmul(a, b)
            e.record()
            e.synchronize()
            best = min(best, s.elapsed_time(e))
        return 2.0 * n ** 3 / (best * 1e-3) / 1e12
    except Exception:
        return None


def make_workload(args):
    """The mid-chain superblock of the chosen configuration (synth.Workload)."""
    from hofstadter_hubbard_tsc_gb300.synth import Workload
    if args.config == "c3":
        return Workload(W=4, L=48, n_elec=176, m=4000, model="tj", J=0.4, phi=1.0 / 6.0)
    if args.config == "c4":
        return Workload(W=6, L=24, n_elec=132, m=6000, U=8.0, phi=1.0 / 3.0)
    return Workload(W=args.W, L=args.L, n_elec=args.ne, m=args.m)


def to_oracle(wl):
    """The workload in the oracle's types (CPU baseline and parity check only)."""
    from oracle import blocks as OB
    from oracle.enlarge import Model
    from oracle.lattice import Lattice

    def blk(b):
        return OB.Block(b.len, b.up_dif, b.down_dif,
                        [OB.Sub(s.num_up, s.num_down, s.down_dif, s.row_dim, s.sdim, s.mat.copy()) for s in b.subs])

    def model(m):
        om = Model(m.len, blk(m.ham))
        om.sub = {i: {n: blk(b) for n, b in d.items()} for i, d in m.sub.items()}
        return om

    def basis(b):
        ob = OB.Basis(b.len)
        for s in b.sectors:
            sec = OB.BSector(s.new_num_up, s.new_num_down)
            for u in s.subs:
                sec.subs.append(OB.BSub(u.spos, u.sdim, u.bl_num_up, u.bl_num_down, u.st_num_up, u.st_num_down))
            sec.dim = s.dim
            ob.sectors.append(sec)
        return ob

    lat = Lattice(wl.W, wl.L, model=wl.model, U=wl.U, J=wl.J, phi=wl.phi)
    sup = OB.Super(wl.sup.sys_len, wl.sup.env_len,
                   [OB.SSector(s.sys_num_up, s.sys_num_down, s.env_num_up, s.env_num_down, s.sys_dim, s.env_dim)
                    for s in wl.sup.subs])
    return model(wl.sys), model(wl.env), basis(wl.sys_bs), basis(wl.env_bs), lat.geometry(wl.sys.len, wl.env.len), sup


def cpu_matvec_timer(wl, psi_flat, nrep):
    """The oracle's model_wave on the workload; returns (seconds per matvec, H psi)."""
    from oracle.matvec import hmerge, model_wave
    from oracle.blocks import allocate_wave
    from oracle.sites import SiteOps
    sys_, env, sbs, ebs, geo, sup = to_oracle(wl)
    hmerge(sys_, env, geo)
    st = SiteOps(wl.model)
    vin = allocate_wave(sup)
    vin.set_flat(psi_flat)
    vout = allocate_wave(sup)
    t0 = time.perf_counter()
    for _ in range(nrep):
        model_wave(sys_, env, sbs, ebs, vin, vout, geo, st)
    dt = (time.perf_counter() - t0) / nrep
    return dt, vout.flat()


def sweep_bench(dev, args):
    """Sweep time on the plain-method lattice: Hubbard 2x16 ladder, phi = 1/4
    (Landau gauge), t = 1, U = 8, N_e = 28 (1/8 hole doping), singlet, Lanczos
    tol 1e-10, at m = 256 (the plain-method configuration) and m = 512 kept
    multiplets.  For each m the warm-up and the two half sweeps run once (split
    precision, untimed) and are checkpointed through the reference's on-disk
    formats; the FP64 arm and the split-precision arm with the learned guess
    corrector are both restored from that checkpoint and time one finite sweep
    each.  The split solver iterates on the tensor-core matvec to 1e-8, its
    noise floor, then restarts with one FP64 product.  The corrector trains
    between sweeps, outside the sweep timer."""
    import shutil
    import tempfile
    from hofstadter_hubbard_tsc_gb300 import _lib
    from hofstadter_hubbard_tsc_gb300.lattice import SquareLattice
    from hofstadter_hubbard_tsc_gb300.sweep import GPUDMRG
    from hofstadter_hubbard_tsc_gb300.guess import LearnedGuess
    lat = SquareLattice(2, 16, U=8.0, phi=0.25)
    nstep = 2 * (lat.N - 3)
    split = PREC[args.sweep_precision]
    results = {}
    for m in args.sweep_m:
        kw = dict(kept_min=m, kept_max=m, trun_err=1e-12, lanzero=1e-10, seed=11)
        hook = LearnedGuess(dev, lat.N, 28)
        prep = GPUDMRG(dev, lat, 28, precision=split, guess_hook=hook, **kw)
        t0 = time.perf_counter()
        prep.run(sweeps=0)
        prep_s = time.perf_counter() - t0
        ckpt = tempfile.mkdtemp(prefix="hh_ckpt_")
        try:
            prep.save(ckpt)
            out = {"config": f"hubbard-ladder-2x16-phi0.25-U8-Ne28-m{m}", "prepare_s": round(prep_s, 3),
                   "split_precision": args.sweep_precision,
                   "start": "warm-up + two half sweeps in split precision, checkpointed and restored by both arms"}
            for name, prec in (("fp64", _lib.HH_PREC_FP64), ("split", split)):
                d = GPUDMRG(dev, lat, 28, precision=prec, guess_hook=hook if name == "split" else None, **kw)
                d.load(ckpt)
                d.phase_s.clear()
                import torch
                torch.cuda.nvtx.range_push(f"sweep_{name}_m{m}")  # profiler filter for the timed sweep
                t0 = time.perf_counter()
                d.sweep()
                dt = time.perf_counter() - t0
                torch.cuda.nvtx.range_pop()
                its = [r[3] for r in d.energies[-nstep:]]
                out[name] = {"E0": d.energies[-1][2], "sweep_s": dt,
                             "lanczos_iterations": int(np.sum(its)), "lanzero": 1e-10,
                             "phase_s": {k: round(v, 4) for k, v in d.phase_s.items()}}
            out["split"]["learned_guess"] = {
                "samples": int(len(hook.data()[1])), "train_s": round(hook.train_s, 4),
                "held_out_hellinger_corrected": hook.val[0] if hook.val else None,
                "held_out_hellinger_plain": hook.val[1] if hook.val else None,
                "applied": bool(hook.enabled), "corrected_steps": int(sum(1 for r in hook.log if r[2]))}
            out["rel_dE"] = abs(out["split"]["E0"] - out["fp64"]["E0"]) / abs(out["fp64"]["E0"])
            out["sweep_speedup_split_vs_fp64"] = out["fp64"]["sweep_s"] / out["split"]["sweep_s"]
            results[f"m{m}"] = out
        finally:
            shutil.rmtree(ckpt, ignore_errors=True)
            hook.free()
    return results


def window_bench(dev, args):
    """Sweep window at the headline configuration: the W = 4, L = 32 cylinder,
    phi = 1/4 (Landau gauge), t = 1, U = 8, N_e = 112 (1/8 hole doping),
    singlet, m kept multiplets (2000), Lanczos tol 1e-10.

    The infinite-system warm-up (warm_up_point, code/warm_up.f90:1284-1491)
    grows both blocks to the middle of the cylinder at m in split precision,
    untimed, and one left-to-right step moves the system block to the middle.
    That state is copied in device memory (the models, truncations and bases
    are shared, immutable handles; the wave is copied).  Each arm -- plain FP64,
    and split precision with the learned guess corrector -- restarts from the
    copy and runs the same K steps of left_to_right (code/warm_up.f90:1495-1671),
    each from the transformed guess of the step before, timed on the host with
    the device synchronised on both sides.  The corrector has no earlier sweep
    to learn from here, so it records and stays on the plain guess.  Riding on
    the FP64 arm, untimed, every step's superblock is also solved by the split
    Lanczos from the same start vector (the precisions compared on one
    superblock and kept basis, step by step)."""
    from hofstadter_hubbard_tsc_gb300 import _lib
    from hofstadter_hubbard_tsc_gb300.device import DWave
    from hofstadter_hubbard_tsc_gb300.lattice import SquareLattice
    from hofstadter_hubbard_tsc_gb300.sweep import GPUDMRG
    from hofstadter_hubbard_tsc_gb300.guess import LearnedGuess
    L, m, K = args.window_L, args.window_m, args.window_steps
    ne = int(round(3.5 * L))
    lat = SquareLattice(4, L, U=8.0, phi=0.25)
    N = lat.N
    split = PREC[args.precision] if args.precision != "fp64" else PREC["bf16x3"]
    kw = dict(kept_min=m, kept_max=m, trun_err=1e-12, lanzero=1e-10, seed=11)
    hook = LearnedGuess(dev, N, ne)
    d = GPUDMRG(dev, lat, ne, precision=split, guess_hook=hook, **kw)
    dev.sync()
    t0 = time.perf_counter()
    d.warm_up()
    d.left_to_right(N // 2 - 1, N // 2)
    dev.sync()
    grow_s = time.perf_counter() - t0
    grow_phase = {k: round(v, 3) for k, v in d.phase_s.items()}
    grow_steps = len(d.energies)

    def copy_wave(wave):
        wv, sup = wave
        w2 = DWave(dev, wv.layout, wv.sys_len, wv.env_len)
        dev.check(dev.lib.hh_wave_copy(w2.h, wv.h))
        return w2, sup

    snap = (dict(d.sys_models), dict(d.env_models), dict(d.sys_truns), dict(d.env_truns), dict(d.sys_bases),
            dict(d.env_bases), copy_wave(d.wave), len(d.energies))

    class SameSuperblock:
        """Rides on the FP64 arm (its time is taken out of that arm's): every
        step's superblock is solved a second time by the split-precision
        Lanczos from the same start vector, so each step compares the two
        precisions on one superblock and one kept basis."""

        def __init__(self):
            self.start, self.E, self.seconds = None, [], 0.0

        def __call__(self, dmrg, sb, psi, when):
            t0 = time.perf_counter()
            if when == "before":
                self.start = DWave(dev, psi.layout, psi.sys_len, psi.env_len)
                dev.check(dev.lib.hh_wave_copy(self.start.h, psi.h))
            else:
                e, _ = sb.lanczos_device(self.start, dmrg.lanzero, dmrg.maxit, precision=split)
                self.E.append(e)
                self.start.free()
            dev.sync()
            self.seconds += time.perf_counter() - t0

    same = SameSuperblock()
    out = {"config": f"hubbard-cylinder-4x{L}-phi0.25-U8-Ne{ne}-m{m}-midchain-window", "steps": K,
           "lanzero": 1e-10, "split_precision": args.precision if args.precision != "fp64" else "bf16x3",
           "start": f"infinite-system warm-up to the middle + 1 left-to-right step in split precision "
                    f"({grow_steps} steps, {grow_s:.1f} s, untimed), copied in device memory for both arms",
           "grow_s": round(grow_s, 2), "grow_phase_s": grow_phase}
    for name, prec in (("fp64", _lib.HH_PREC_FP64), ("split", split)):
        d.sys_models = {k: v.copy() for k, v in snap[0].items()}
        d.env_models = {k: v.copy() for k, v in snap[1].items()}
        d.sys_truns, d.env_truns, d.sys_bases, d.env_bases = (dict(snap[2]), dict(snap[3]), dict(snap[4]),
                                                              dict(snap[5]))
        d.wave = copy_wave(snap[6])
        del d.energies[snap[7]:]
        d.precision = prec
        d.guess_hook = hook if name == "split" else same
        d.phase_s.clear()
        dev.sync()
        t0 = time.perf_counter()
        d.left_to_right(N // 2, N // 2 + K)
        dev.sync()
        dt = time.perf_counter() - t0
        if name == "fp64":  # the same-superblock solves are not the FP64 arm's work
            dt -= same.seconds
            d.phase_s.pop("guess", None)
        steps = d.energies[-K:]
        out[name] = {"window_s": dt, "s_per_step": dt / K, "E0": [e[2] for e in steps],
                     "lanczos_iterations": [int(e[3]) for e in steps],
                     "phase_s": {k: round(v, 4) for k, v in d.phase_s.items()},
                     "kept": int(d.last_trunc[0]) if hasattr(d, "last_trunc") else None}
    out["split"]["learned_guess"] = {"samples": int(len(hook.data()[1])), "applied": bool(hook.enabled),
                                     "note": "no earlier sweep to train on inside the window"}
    e64, esp = np.array(out["fp64"]["E0"]), np.array(out["split"]["E0"])
    out["rel_dE_per_step"] = (np.abs(esp - e64) / np.abs(e64)).tolist()
    out["rel_dE"] = float(np.max(out["rel_dE_per_step"]))
    # the first step solves the same superblock in both arms (the solver's
    # precision); later steps follow each arm's own truncations, whose kept
    # bases move with the converged vector within the Lanczos tolerance
    out["rel_dE_first_step"] = out["rel_dE_per_step"][0]
    # every step's FP64 superblock solved again in split precision, same start
    out["rel_dE_same_superblock_per_step"] = (np.abs(np.array(same.E) - e64) / np.abs(e64)).tolist()
    out["rel_dE_same_superblock"] = float(np.max(out["rel_dE_same_superblock_per_step"]))
    out["same_superblock_check_s"] = round(same.seconds, 3)
    out["sweep_speedup_split_vs_fp64"] = out["fp64"]["window_s"] / out["split"]["window_s"]
    hook.free()
    d.sys_models = d.env_models = d.sys_truns = d.env_truns = d.sys_bases = d.env_bases = {}
    d.wave = None
    return out


def config_matvec_bench(dev, name, steps, prec_name):
    """The matvec of another configuration's mid-chain superblock (c3: t-J 4x48,
    J = 0.4, phi = 1/6, N_e = 176, m = 4000; c4: Hubbard 6x24, phi = 1/3, U = 8,
    N_e = 132, m = 6000; synthetic operators as for the headline workload):
    split-precision matvecs/s by CUDA events over `steps` graph replays (L2
    flushed before each), the FP64 GPU matvec rate over one product, and the
    split product's error against FP64."""
    import ctypes as C
    import torch
    from hofstadter_hubbard_tsc_gb300.superblock import Superblock
    from hofstadter_hubbard_tsc_gb300 import _lib
    a = argparse.Namespace(config=name, W=4, L=32, ne=112, m=2000)
    t0 = time.perf_counter()
    wl = make_workload(a)
    gen_s = time.perf_counter() - t0
    prec = PREC[prec_name]
    dev.sync()
    t0 = time.perf_counter()
    sb = Superblock(dev, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo, precision=prec)
    dev.sync()
    plan_s = time.perf_counter() - t0
    rng = np.random.default_rng(5)
    psi = rng.normal(size=wl.sup.dim) + 1j * rng.normal(size=wl.sup.dim)
    psi /= np.linalg.norm(psi)
    sb.w_in.upload(psi)
    stream = torch.cuda.ExternalStream(dev.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(pp, n):
        for _ in range(2):
            dev.check(dev.lib.hh_matvec_async(sb.plan, sb.w_in.h, sb.w_out.h, pp))
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        with torch.cuda.stream(stream):
            for e0, e1 in ev:
                flush.zero_()
                e0.record(stream)
                dev.check(dev.lib.hh_matvec_async(sb.plan, sb.w_in.h, sb.w_out.h, pp))
                e1.record(stream)
        dev.check(dev.lib.hh_plan_check(sb.plan))
        torch.cuda.synchronize()
        return sum(e0.elapsed_time(e1) for e0, e1 in ev) / n

    tune = None
    if prec != _lib.HH_PREC_FP64:  # the schedule autotuner on this workload
        tms, tch = np.zeros(_lib.HH_TUNE_VARIANTS), C.c_int(0)
        t0 = time.perf_counter()
        dev.check(dev.lib.hh_plan_tune(sb.plan, prec, 2, tms.ctypes.data_as(C.POINTER(C.c_double)), C.byref(tch)))
        tune = {"variants_ms": [round(x, 4) for x in tms], "chosen": int(tch.value),
                "tune_s": round(time.perf_counter() - t0, 3)}
    ms_split = timed(prec, steps)
    hs = sb.w_out.download()
    dev.check(dev.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, _lib.HH_PREC_FP64))
    h64 = sb.w_out.download()
    ms64 = timed(_lib.HH_PREC_FP64, 1)
    out = {"config": dict(wl.describe(), **{"precision": prec_name}), "matvecs_per_s": 1e3 / ms_split,
           "ms_per_matvec": ms_split, "steps": steps, "fp64_matvecs_per_s": 1e3 / ms64,
           "split_vs_fp64_matvec": ms64 / ms_split,
           "rel_err_vs_fp64_gpu": float(np.linalg.norm(hs - h64) / np.linalg.norm(h64)),
           "workload_generation_s": round(gen_s, 2), "plan_build_s": round(plan_s, 3), "autotune": tune,
           "timing": "CUDA events on the library stream, graph replays, L2 flushed before each"}
    sb.free()
    del flush
    return out


def run_c5(args, local):
    """The synthetic block-sparse matvec: a mid-chain superblock of the 6-wide
    cylinder (phi = 1/3, U = 8, N_e = 132: the 12-term Hamiltonian) whose
    blocks have 150 SU(2) sectors each with lognormal dimensions (median 96,
    maximum 2048, seeded), N(0,1) operators, and 8 uneven wavefunctions
    (per-sector lognormal weights, norms over eight decades) multiplied in
    one graph replay (every stage one launch over the batch).  Reported:
    vectors/s of the batched replay (CUDA events, L2 flushed before each
    step), the same 8 vectors one replay each, the FP64 GPU product, and the
    split product's error against FP64 for two of the vectors."""
    import ctypes as C
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from hofstadter_hubbard_tsc_gb300 import _lib
    from hofstadter_hubbard_tsc_gb300.device import Device, DWave
    from hofstadter_hubbard_tsc_gb300.superblock import Superblock
    from hofstadter_hubbard_tsc_gb300.synth import Workload, uneven_batch
    torch.cuda.set_device(local)
    nb = 8
    prec = PREC[args.precision]
    t0 = time.perf_counter()
    wl = Workload(W=6, L=24, n_elec=132, U=8.0, phi=1.0 / 3.0, lognormal=(150, 96, 2048))
    psi = uneven_batch([s.sys_dim * s.env_dim for s in wl.sup.subs], nb, np.random.default_rng(4))
    gen_s = time.perf_counter() - t0
    dev = Device(local)
    dev.sync()
    t0 = time.perf_counter()
    sb = Superblock(dev, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo, precision=prec)
    dev.sync()
    plan_s = time.perf_counter() - t0
    lay = sb.w_in.layout
    win = DWave(dev, lay, sb.w_in.sys_len, sb.w_in.env_len, nbatch=nb)
    wout = DWave(dev, lay, sb.w_in.sys_len, sb.w_in.env_len, nbatch=nb)
    win.upload(psi)
    stream = torch.cuda.ExternalStream(dev.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed(fn, n):
        for _ in range(max(args.warmup, 3)):
            fn()
        dev.check(dev.lib.hh_plan_check(sb.plan))
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        with torch.cuda.stream(stream):
            for e0, e1 in ev:
                flush.zero_()
                e0.record(stream)
                fn()
                e1.record(stream)
        dev.check(dev.lib.hh_plan_check(sb.plan))
        torch.cuda.synchronize()
        return sum(e0.elapsed_time(e1) for e0, e1 in ev) / n

    t0 = time.perf_counter()
    dev.check(dev.lib.hh_matvec(sb.plan, win.h, wout.h, prec))  # builds the batch schedule
    dev.sync()
    batch_setup_s = time.perf_counter() - t0
    clocks = Clocks(local)
    clocks.start()
    ms_batch = timed(lambda: dev.check(dev.lib.hh_matvec_async(sb.plan, win.h, wout.h, prec)), args.steps)
    clk = clocks.stop()
    got = wout.download().reshape(nb, -1)

    sb.w_in.upload(psi[0])
    ms_single = timed(lambda: dev.check(dev.lib.hh_matvec_async(sb.plan, sb.w_in.h, sb.w_out.h, prec)),
                      max(2, args.steps // 2))
    errs = {}
    t64 = None
    for b in (0, nb - 1):
        sb.w_in.upload(psi[b])
        dev.sync()
        t0 = time.perf_counter()
        dev.check(dev.lib.hh_matvec(sb.plan, sb.w_in.h, sb.w_out.h, _lib.HH_PREC_FP64))
        dev.sync()
        t64 = time.perf_counter() - t0
        h64 = sb.w_out.download()
        errs[b] = float(np.linalg.norm(got[b] - h64) / np.linalg.norm(h64))
    counts = np.zeros(_lib.HH_PLAN_STATS)
    dev.check(dev.lib.hh_plan_stats(sb.plan, counts.ctypes.data_as(C.POINTER(C.c_double))))
    peaks = measured_peaks()
    nprod = 6 if prec == _lib.HH_PREC_BF16X6 else 3
    achieved = nb * counts[1] / (ms_batch * 1e-3) / 1e12
    peak = peaks["bf16_tflops"] / nprod
    value = nb / (ms_batch * 1e-3)
    line = {"metric": METRIC, "value": value, "unit": "vectors/s (matvecs/s over the 8-vector batch)",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_batch,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": f"{args.precision}(c128 io)", "data": "synthetic",
            "config": dict(wl.describe(), **{"workload": "synthetic-block-sparse-300-sectors-lognormal96-max2048-"
                                                         "12terms-8psi", "batch": nb, "precision": args.precision,
                                             "l2": "flushed between steps (256 MB write)",
                                             "matvec_launch": "one CUDA-graph replay per step for all 8 vectors"}),
            "gpu_launches": int(args.steps * counts[17]),
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None,
                         "kernel": "whole batched matvec (wave images, stage 1, stage 2, copy terms)",
                         "peak_note": f"measured bf16 burst / {nprod}",
                         "algorithmic_flops_per_launch": nb * counts[1]},
            "vector_by_vector": {"value": 1e3 / ms_single, "ms_per_vector": ms_single,
                                 "batch_speedup": (1e3 / ms_single) and value / (1e3 / ms_single)},
            "fp64_gpu": {"value": 1.0 / t64 if t64 else None, "unit": "vectors/s", "s_per_vector": t64},
            "rel_err_vs_fp64_gpu": errs, "clocks": clk,
            "e2e": None, "e2e_note": "the batched entry point takes device waves; the host-buffer call is "
                                      "single-vector (hh_matvec_host)",
            "setup_s": {"workload_generation": round(gen_s, 1), "plan": round(plan_s, 2),
                        "batch_schedule_and_first_replay": round(batch_setup_s, 2)},
            "ref_gflop_per_vector": counts[0] / 1e9, "exec_gflop_per_vector": counts[1] / 1e9}
    print(json.dumps(line), flush=True)
    del flush
    win.free()
    wout.free()
    sb.free()
    dev.close()


def run_reference(args, rank, ws, dist):
    if rank != 0:
        return
    wl = make_workload(args)
    rng = np.random.default_rng(1)
    psi = rng.normal(size=wl.sup.dim) + 1j * rng.normal(size=wl.sup.dim)
    steps = max(1, args.steps)
    for _ in range(args.warmup):
        cpu_matvec_timer(wl, psi, 1)
    dt, _ = cpu_matvec_timer(wl, psi, steps)
    v = 1.0 / dt
    cores = os.cpu_count()
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": dict(wl.describe(), **{"timing": "host wall clock per matvec"}),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{steps} full matvec(s) of the workload (numpy restatement of model_wave, "
                                       f"OpenBLAS threads = all host cores)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    dist, rank, ws, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, rank, ws, dist)
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return
    if args.config == "c5":
        run_c5(args, local)
        return
    import ctypes as C
    import torch
    torch.cuda.set_device(local)
    import __graft_entry__
    __graft_entry__.build()
    from hofstadter_hubbard_tsc_gb300 import _lib
    from hofstadter_hubbard_tsc_gb300.device import Device, DWave
    from hofstadter_hubbard_tsc_gb300.superblock import Superblock

    prec = PREC[args.precision]
    t0 = time.perf_counter()
    wl = make_workload(args)
    workload_s = time.perf_counter() - t0
    dev = Device(local)
    dev.check(dev.lib.hh_ctx_set_eigensolver(dev.h, _lib.HH_EIG_OWN if args.eigensolver == "own"
                                             else _lib.HH_EIG_CUSOLVER))
    # host-side cost of one superblock at this size: operator upload, hmerge
    # and the task list (hh_plan_create), then the split-precision schedule
    # and operator images, built by the first split-precision matvec
    dev.sync()
    t0 = time.perf_counter()
    sb = Superblock(dev, wl.sys, wl.env, wl.sys_bs, wl.env_bs, wl.sup, wl.geo, precision=prec)
    dev.sync()
    plan_build_s = time.perf_counter() - t0
    stats = sb.stats()
    rng = np.random.default_rng(1 + rank)
    psi = rng.normal(size=wl.sup.dim) + 1j * rng.normal(size=wl.sup.dim)
    psi /= np.linalg.norm(psi)
    w_in, w_out = sb.w_in, sb.w_out
    w_in.upload(psi)
    image_build_s = None
    if prec != _lib.HH_PREC_FP64:
        dev.sync()
        t0 = time.perf_counter()
        dev.check(dev.lib.hh_matvec(sb.plan, w_in.h, w_out.h, prec))
        dev.sync()
        image_build_s = time.perf_counter() - t0

    stream = torch.cuda.ExternalStream(dev.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > 129 MB L2
    ms = (C.c_float * 4)()

    # schedule autotuner (split precision): stage-2 tile shape x stage 1 / stage 2
    # persistent or per tile
    tune_ms, tune_choice = np.zeros(_lib.HH_TUNE_VARIANTS), C.c_int(0)
    t0 = time.perf_counter()
    dev.check(dev.lib.hh_plan_tune(sb.plan, prec, 3, tune_ms.ctypes.data_as(C.POINTER(C.c_double)),
                                   C.byref(tune_choice)))
    tune_s = time.perf_counter() - t0

    def staged():
        dev.check(dev.lib.hh_matvec_timed(sb.plan, w_in.h, w_out.h, prec, ms))
        return ms[0], ms[1], ms[2], ms[3]

    # timed steps: the user-facing matvec (hh_matvec_async: one CUDA-graph
    # replay on the library's stream), CUDA events on that stream, L2 flushed
    # before each step outside the event window
    for _ in range(max(args.warmup, 3)):
        dev.check(dev.lib.hh_matvec_async(sb.plan, w_in.h, w_out.h, prec))
    dev.check(dev.lib.hh_plan_check(sb.plan))
    if dist:
        dist.barrier()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = Clocks(local)
    clocks.start()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed")
    with torch.cuda.stream(stream):
        for a, b in ev:
            flush.zero_()
            a.record(stream)
            dev.check(dev.lib.hh_matvec_async(sb.plan, w_in.h, w_out.h, prec))
            b.record(stream)
    dev.check(dev.lib.hh_plan_check(sb.plan))
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    clk = clocks.stop()
    tot = sum(a.elapsed_time(b) for a, b in ev)
    # per-stage device times of the same matvec launched eagerly with events
    # between the stages (same flush), for the roofline of the dominant kernel
    s1 = s2 = s0 = sc = 0.0
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        a, b, c, d = staged()
        s1 += b
        s2 += c
        s0 += d
        sc += max(0.0, a - b - c - d)  # the copy terms after the stage-2 tiles
    t_steps = max_over_ranks(tot / 1e3, dist, "cuda")  # seconds, device time of the K matvecs
    value = replica_rate(ws, args.steps, t_steps)

    # end to end through the C-ABI call with pinned host buffers
    nbytes = wl.sup.dim * 16
    hin, hout = C.c_void_p(), C.c_void_p()
    dev.check(dev.lib.hh_host_alloc(nbytes, C.byref(hin)))
    dev.check(dev.lib.hh_host_alloc(nbytes, C.byref(hout)))
    hin_np = np.ctypeslib.as_array((C.c_double * (2 * wl.sup.dim)).from_address(hin.value))
    hout_np = np.ctypeslib.as_array((C.c_double * (2 * wl.sup.dim)).from_address(hout.value))
    hin_np[:] = psi.view(np.float64)
    dp = C.POINTER(C.c_double)
    for _ in range(max(1, args.warmup)):
        dev.check(dev.lib.hh_matvec_host(sb.plan, C.cast(hin, dp), C.cast(hout, dp), prec))
    if dist:
        dist.barrier()
    te = time.perf_counter()
    for _ in range(args.steps):
        dev.check(dev.lib.hh_matvec_host(sb.plan, C.cast(hin, dp), C.cast(hout, dp), prec))
    te = time.perf_counter() - te
    if dist:
        t = torch.tensor([te], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        te = float(t.item())
    hpsi_gpu = hout_np.view(np.complex128).copy()
    e2e = {"value": ws * args.steps / te, "unit": UNIT, "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
           "timing": "host wall clock around hh_matvec_host (pinned H2D, matvec, D2H, stream sync)"}

    # roofline of the dominant kernel (the stage with more device time)
    peaks = measured_peaks()
    stage = 1 if s1 >= s2 else 2
    t_stage = (s1 if stage == 1 else s2) / args.steps * 1e-3
    counts = np.zeros(_lib.HH_PLAN_STATS)
    dev.check(dev.lib.hh_plan_stats(sb.plan, counts.ctypes.data_as(dp)))
    flops_stage = counts[8] if stage == 1 else counts[9]
    achieved = flops_stage / t_stage / 1e12
    if prec == _lib.HH_PREC_FP64:
        peak = fp64_peak_tflops()
        peak_note = "dense FP64 (cuBLAS DGEMM 4096^3, best of 5, measured in this run): GB300 has no FP64 tensor path"
    else:
        nprod = 6 if prec == _lib.HH_PREC_BF16X6 else 3
        peak = peaks["bf16_tflops"] / nprod
        peak_note = (f"measured bf16 burst / {nprod} ({args.precision}: {nprod} bf16 products per real product)")
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": (achieved / peak) if peak else None,
                "traffic": (captured_traffic(wl.describe()["workload"], args.precision)
                            if stage == 2 and prec != _lib.HH_PREC_FP64 else None),
                "kernel": (f"seg_gemm_fp64 stage {stage}" if prec == _lib.HH_PREC_FP64
                           else f"tc_tile_kernel stage {stage} (the tile kernel alone; copy terms in stage_ms)"),
                "peak_note": peak_note,
                "algorithmic_flops_per_launch": flops_stage,
                "kernel_ms_per_launch": t_stage * 1e3}
    if prec != _lib.HH_PREC_FP64:
        issued = (counts[12] if stage == 1 else counts[13]) * (1.0 if prec == _lib.HH_PREC_BF16X6 else 0.5)
        roofline["bf16_flops_issued_per_launch"] = issued
        roofline["tensor_pipe_frac_of_measured_bf16"] = issued / t_stage / 1e12 / peaks["bf16_tflops"]
        if stage == 2:
            # the tile list's own MMA floor: its MMA cycles (max(45, width/2)
            # per K = 16 MMA, measured) spread evenly over every SM's tensor core
            sms = torch.cuda.get_device_properties(0).multi_processor_count
            mhz = (clk or {}).get("sm_mhz") or 2070.0
            cyc = counts[22] * (2.0 if prec == _lib.HH_PREC_BF16X6 else 1.0)
            floor_ms = cyc / sms / (mhz * 1e6) * 1e3
            roofline["stage2_tiles"] = {"tiles": int(counts[20]), "stacked": int(counts[21]),
                                        "tile_shape": int(counts[23]), "mma_cycle_floor_ms": floor_ms,
                                        "kernel_over_floor": t_stage * 1e3 / floor_ms if floor_ms else None}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "c128" if prec == _lib.HH_PREC_FP64 else f"{args.precision}(c128 io)",
            "data": "synthetic",
            "config": dict(wl.describe(), **{"precision": args.precision, "l2": "flushed between steps (256 MB write)",
                                             "density_eigensolver": args.eigensolver,
                                             "parallelism": f"replicas x{ws}",
                                             "matvec_launch": ("one CUDA-graph replay per step (hh_matvec_async)"
                                                               if prec != _lib.HH_PREC_FP64 else "eager"),
                                             "autotune": ({"variants_ms": [round(x, 4) for x in tune_ms],
                                                           "variant_index": "4*stage2_tile_shape+2*stage1_persistent+stage2_persistent",
                                                           "chosen": int(tune_choice.value), "tune_s": round(tune_s, 3)}
                                                          if prec != _lib.HH_PREC_FP64 else None),
                                             "ref_gflop_per_matvec": counts[0] / 1e9,
                                             "exec_gflop_per_matvec": counts[1] / 1e9,
                                             "workload_generation_s": round(workload_s, 3)}),
            "plan_build_s": plan_build_s,
            "image_build_s": image_build_s,
            "roofline": roofline, "e2e": e2e, "clocks": clk,
            "stage_ms": {"wave_images": s0 / args.steps, "stage1": s1 / args.steps,
                         "stage2": s2 / args.steps, "copy_terms": sc / args.steps},
            "gpu_launches": int(args.steps * (counts[16] if prec == _lib.HH_PREC_FP64 else counts[17]))}
    if prec != _lib.HH_PREC_FP64:
        w_in.upload(psi)
        dev.check(dev.lib.hh_matvec(sb.plan, w_in.h, w_out.h, _lib.HH_PREC_FP64))
        h64 = w_out.download()
        dev.check(dev.lib.hh_matvec(sb.plan, w_in.h, w_out.h, prec))
        hmx = w_out.download()
        line["rel_err_vs_fp64_gpu"] = float(np.linalg.norm(hmx - h64) / np.linalg.norm(h64))
        # the FP64 GPU path on the same workload (the metric's comparison arm):
        # CUDA events on the library's stream, L2 flushed before each matvec
        n64 = 3
        ev64 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n64)]
        with torch.cuda.stream(stream):
            for a, b in ev64:
                flush.zero_()
                a.record(stream)
                dev.check(dev.lib.hh_matvec_async(sb.plan, w_in.h, w_out.h, _lib.HH_PREC_FP64))
                b.record(stream)
        dev.check(dev.lib.hh_plan_check(sb.plan))
        t64 = sum(a.elapsed_time(b) for a, b in ev64) / n64
        line["fp64_gpu"] = {"value": 1e3 / t64, "unit": UNIT, "ms_per_step": t64, "steps": n64,
                            "split_vs_fp64_matvec": (1e3 / t64) and value / (1e3 / t64)}
        # the double-float product (the split Lanczos's restart product):
        # rate and error against FP64, same timing
        dev.check(dev.lib.hh_matvec(sb.plan, w_in.h, w_out.h, _lib.HH_PREC_FP32X2))
        hdf = w_out.download()
        evd = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n64)]
        with torch.cuda.stream(stream):
            for a, b in evd:
                flush.zero_()
                a.record(stream)
                dev.check(dev.lib.hh_matvec_async(sb.plan, w_in.h, w_out.h, _lib.HH_PREC_FP32X2))
                b.record(stream)
        dev.check(dev.lib.hh_plan_check(sb.plan))
        tdf = sum(a.elapsed_time(b) for a, b in evd) / n64
        line["fp32x2_gpu"] = {"value": 1e3 / tdf, "unit": UNIT, "ms_per_step": tdf, "steps": n64,
                              "vs_fp64_gpu": t64 / tdf,
                              "rel_err_vs_fp64_gpu": float(np.linalg.norm(hdf - h64) / np.linalg.norm(h64))}
    if prec != _lib.HH_PREC_FP64:
        # 8 vectors of the same workload in one graph replay (every stage one
        # launch over the batch) against the single-vector replays above
        nbt = 8
        wbi = DWave(dev, w_in.layout, w_in.sys_len, w_in.env_len, nbatch=nbt)
        wbo = DWave(dev, w_in.layout, w_in.sys_len, w_in.env_len, nbatch=nbt)
        rb = np.random.default_rng(11)
        wbi.upload(rb.normal(size=(nbt, wl.sup.dim)) + 1j * rb.normal(size=(nbt, wl.sup.dim)))
        dev.check(dev.lib.hh_matvec(sb.plan, wbi.h, wbo.h, prec))
        for _ in range(3):
            dev.check(dev.lib.hh_matvec_async(sb.plan, wbi.h, wbo.h, prec))
        evb = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        with torch.cuda.stream(stream):
            for a, b in evb:
                flush.zero_()
                a.record(stream)
                dev.check(dev.lib.hh_matvec_async(sb.plan, wbi.h, wbo.h, prec))
                b.record(stream)
        dev.check(dev.lib.hh_plan_check(sb.plan))
        torch.cuda.synchronize()
        tb = sum(a.elapsed_time(b) for a, b in evb) / args.steps
        line["batched_8"] = {"value": nbt * 1e3 / tb, "unit": "vectors/s", "ms_per_replay": tb,
                             "vs_single_vector_replays": nbt * 1e3 / tb / value,
                             "timing": "CUDA events, one graph replay for 8 vectors, L2 flushed before each"}
        wbi.free()
        wbo.free()
    if rank == 0 and not args.no_sweep and args.config == "c2":
        line["sweep"] = sweep_bench(dev, args)
    if rank == 0 and not args.no_window and args.config == "c2":
        line["sweep_window"] = window_bench(dev, args)
    if rank == 0 and not args.no_configs and args.config == "c2":
        line["other_configs"] = {name: config_matvec_bench(dev, name, 5, args.precision) for name in ("c3", "c4")}
    if not args.no_energy_check:
        rs = np.random.default_rng(7)
        start = rs.normal(size=wl.sup.dim) + 1j * rs.normal(size=wl.sup.dim)
        res = {}
        for name, pp in (("fp64", _lib.HH_PREC_FP64), ("split", prec)):
            w_in.upload(start)
            e, it = C.c_double(), C.c_int()
            t0 = time.perf_counter()
            dev.check(dev.lib.hh_lanczos(sb.plan, w_in.h, 1e-12, 100, pp, C.byref(e), C.byref(it)))
            res[name] = (e.value, it.value, time.perf_counter() - t0)
        line["energy_check"] = {"E_fp64": res["fp64"][0], "E_split": res["split"][0],
                                "rel_dE": abs(res["split"][0] - res["fp64"][0]) / abs(res["fp64"][0]),
                                "iterations": [res["fp64"][1], res["split"][1]],
                                "lanczos_s": [res["fp64"][2], res["split"][2]]}
    if rank == 0 and not args.no_cpu_baseline:
        n = max(1, args.cpu_sample)
        dt, hpsi_cpu = cpu_matvec_timer(wl, psi, n)
        rel = float(np.linalg.norm(hpsi_gpu - hpsi_cpu) / np.linalg.norm(hpsi_cpu))
        line["cpu_baseline"] = {"value": 1.0 / dt, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{n} full matvec(s) of the same workload (numpy restatement of "
                                          f"model_wave, OpenBLAS on all host cores)",
                                "achieved_gflops": counts[0] / 1e9 / dt,
                                "gflops_note": "reference FLOPs of the matvec (8MNK over its ZGEMM calls + 8 per "
                                               "copied element) / wall time"}
        line["parity_rel_err_vs_oracle"] = rel
    if rank == 0:
        print(json.dumps(line), flush=True)
    sb.free()
    dev.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
