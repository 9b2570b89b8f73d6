"""Benchmark of the fix-eph hot path on GB300: fix-eph atom-steps/s.

Workload (the plain cascade at scale): fcc Ni 80x80x80 cells (2,048,000
atoms) at 300 K, a 10 keV primary knock-on atom at the box centre, dt 0.5 fs,
the synthetic beta file (rho(r) = exp(-r/0.6) cut at 4.6 A, beta(rho) = 0.05
+ 0.02 tanh(rho - 2), 2,000 knots each), flags 7 (friction + random + FDM),
model 4, FDM grid 64^3 with C_e 3.5e-6, kappa 0.1, T_e 300 K.  Seeded synthetic
inputs stand in for the reference's LAMMPS decks; no pair potential (the metric
excludes pair forces: external force zero).

One step = one engine step through the fix: initial_integrate, position wrap
check, binning + in-cutoff pair list (kept candidate lists), density,
friction pre-vector, friction + random forces, final_integrate, energy
deposition, FDM substeps; FAST mode, the per-atom work in FP64 and the pair
terms in double-float (df64).  `value` is device-resident (CUDA events on the
fix's stream); `e2e` drives the same step through the C ABI hooks the LAMMPS
fix calls, with its host arrays (positions, velocities, forces and the
per-atom array copied in and out every step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "user-eph_gb300"))
sys.path.insert(0, REPO)

CELLS = 80
GRID = (64, 64, 64)
DT = 0.0005
# list skins (A) that --autotune-skin times (0: the bin search every step)
SKIN_CANDIDATES = (0.0, 0.15, 0.2, 0.3, 0.4, 0.6)
PKA_EV = 10000.0
SEED = 4242
WORKLOAD = "fcc Ni 80^3 cells (2,048,000 atoms), 10 keV PKA, dt 0.5 fs, FDM 64^3, flags 7, model 4"
METRIC = "fix-eph atom-steps/s"


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_system(workdir, cells=None, grid=None):
    from ephgb import workloads as W

    cells = CELLS if cells is None else cells
    grid = GRID if grid is None else grid
    bf = W.write_beta_file(os.path.join(workdir, "synth.beta"))
    atoms = W.fcc_lattice(cells, seed=SEED)
    W.add_pka(atoms, PKA_EV, seed=SEED + 1)
    words = W.fix_args(bf, seed=SEED, flags=7, model=4, grid=grid, T_out=os.path.join(workdir, "Te_out"))
    return words, atoms


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for k, name in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def density_bytes(n_atoms, n_pairs):
    """Algorithmic HBM bytes of one launch of the density sweep of the bench
    workload (k_density_list_df: FAST, one element, stage 1 folded, df64 pair
    sums over the kept candidate lists): per atom read x_i, v_i (64 B), mask,
    state, list length (12), the atom's df64 record (32), T_e at the atom (8);
    written pair count (4), A_i, Bw_i (64), M_i (64), G_i (48), rho, beta, T_e
    at the atom (24), cell (4); per in-cutoff pair its list entry read (4) and
    the cached index (4), e_ij and H e as double-floats (48) written.  The
    neighbours' records, the spline table and the list entries of the shell
    beyond the cut-off are not counted."""
    return 324 * n_atoms + 56 * n_pairs


def forces_bytes(n_atoms, n_pairs):
    """Algorithmic HBM bytes of one launch of the force sweep (k_forces_df,
    FAST, one element): per atom its record flag (16 B), pair count (4), A_i,
    Bw_i (64), M_i (64), T_e at the atom (8), f read and written (64), f_EPH
    and f_RNG written (64); per in-cutoff pair the cached index (4), e_ij and
    H e as double-floats (48).  The neighbours' records G_j are not counted."""
    return 284 * n_atoms + 52 * n_pairs


# DRAM bytes of one launch (dram__bytes_read.sum + dram__bytes_write.sum) over
# the algorithmic bytes of that launch, from ncu captures of each kernel
# alone on the 131,072-atom cascade (`bench.py --cells 32 --grid 26`, kept
# lists, 42.0 pairs per atom, like the bench workload); the bench's traffic figure is this ratio times the algorithmic
# bytes at its own size.  Under 1: part of a sweep's pair-cache writes is
# still in L2 when it ends.
DENSITY_DRAM_OVER_ALGORITHMIC = 0.858
FORCES_DRAM_OVER_ALGORITHMIC = 0.987
# pipe and issue figures of the two sweeps (ncu, the same captures)
DENSITY_PIPES = {"issue_active": 0.469, "fma_pipe": 0.332, "alu_pipe": 0.144, "fp64_pipe": 0.294,
                 "top_stall": "long_scoreboard"}
FORCES_PIPES = {"issue_active": 0.379, "fma_pipe": 0.298, "alu_pipe": 0.083, "fp64_pipe": 0.157,
                "top_stall": "long_scoreboard"}


def step_bytes_8d(n_list=78, sweeps=3):
    """Algorithmic HBM bytes of one atom-step by the hot-path scope's own
    count (a stored full list of n_list entries per atom read by `sweeps`
    list sweeps, 4 B each; x, v, type read over the passes, 156 B; xi, T_e
    at the atom, rho, alpha, w, f_EPH, f_RNG, f and the deposition, 224 B):
    1,316 B at n_list = 78 (the list with a 1 A skin) and 3 sweeps."""
    return 4 * n_list * sweeps + 156 + 224


def ranks_reduce(x, op, device):
    """x combined over the ranks of the process group ("max" for times, "sum"
    for throughputs of independent replicas); x itself without a group or
    with one rank."""
    import torch

    if not torch.distributed.is_available() or not torch.distributed.is_initialized():
        return x
    if torch.distributed.get_world_size() == 1:
        return x
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    rop = {"max": torch.distributed.ReduceOp.MAX, "sum": torch.distributed.ReduceOp.SUM}[op]
    torch.distributed.all_reduce(t, op=rop)
    return float(t.item())


def job_value(world, atoms_per_rank, steps, max_ms):
    """Whole-job atom-steps/s: every rank steps its own replica of the
    workload (weak scaling), timed by the slowest rank."""
    return world * atoms_per_rank * steps / (max_ms / 1000.0)


def run_gpu(args, rank, world):
    import torch

    import ephgb

    dev = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(dev)
    out = {}
    with tempfile.TemporaryDirectory() as wd:
        words, atoms = make_system(wd)
        n = atoms.n
        fix = ephgb.FixEPH(words, atoms, dt=DT, mode=ephgb.MODE_FAST, device=dev)
        if args.list_skin is not None:
            fix.set_list_skin(args.list_skin)
        stream = torch.cuda.current_stream()
        fix.set_stream(stream.cuda_stream)
        # ---------------------------------------------- device-resident value
        fix.step(args.warmup)
        fix.synchronize()
        tuned = None
        if args.autotune_skin:
            # eph_autotune_list_skin: trial windows from this state, restored
            tuned = fix.autotune_list_skin(SKIN_CANDIDATES, steps=args.autotune_steps)
            fix.step(2)  # the build of the chosen radius, outside the timed steps
            fix.synchronize()
        if world > 1:
            torch.distributed.barrier()
        builds0 = fix.counter("build")
        fix.set_profiling(True)
        clocks = ClockSampler(dev)
        clocks.start()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fix.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = ranks_reduce(e0.elapsed_time(e1), "max", "cuda")
        clock = clocks.stop()
        fix.synchronize()
        phases = fix.phase_times()
        launches = fix.launch_count()
        fix.set_profiling(False)
        n_pairs = fix.pair_count()
        out.update(ms=ms, phases=phases, launches=launches, n_pairs=n_pairs, clocks=clock, n=n,
                   rebuilds=fix.counter("wrap"), list_builds=fix.counter("build") - builds0, list_skin=fix.list_skin(),
                   skin_autotuned=tuned)
        if not args.no_fp64_pairs:
            # the same steps with the pair terms in FP64 (EPH_PAIRS_FP64), from
            # the state reached: the rate of the FP64-throughout form
            fix.set_pair_arithmetic(ephgb.PAIRS_FP64)
            fix.step(3)
            fix.synchronize()
            k64 = max(1, min(args.steps, 50))
            e0.record(stream)
            fix.step(k64)
            e1.record(stream)
            torch.cuda.synchronize()
            out.update(ms64=ranks_reduce(e0.elapsed_time(e1), "max", "cuda"), steps64=k64)
            fix.set_pair_arithmetic(ephgb.PAIRS_DF64)
            fix.step(2)
            fix.synchronize()
        if args.no_e2e:
            return out
        # ------------------------------------------------ end to end (host)
        x = torch.empty((n, 3), dtype=torch.float64).pin_memory()
        v = torch.empty((n, 3), dtype=torch.float64).pin_memory()
        f = torch.zeros((n, 3), dtype=torch.float64).pin_memory()
        f0_t = torch.zeros((n, 3), dtype=torch.float64).pin_memory()
        x.numpy()[:] = fix.get("x")
        v.numpy()[:] = fix.get("v")
        e2e_steps = max(1, min(args.steps, 20))

        arr_t = torch.zeros((n, 8), dtype=torch.float64).pin_memory()
        xn, vn, fn, f0, arr = x.numpy(), v.numpy(), f.numpy(), f0_t.numpy(), arr_t.numpy()
        step_no = [0]

        def host_step():
            # the hooks of the LAMMPS fix eph/gb (user-eph_gb300/lammps/fix_eph_gb.cpp)
            # with its default settings, on a step where the engine re-neighbours
            # without re-sorting (the knock-on atom moves more than half the skin
            # every step, so LAMMPS rebuilds its lists every step here):
            step_no[0] += 1
            # initial_integrate: x, v in, the half kick and drift, x, v out
            # (the device keeps the f final_integrate sent)
            fix.initial_integrate_host(xn, vn)
            # post_force after the engine's re-neighbouring: x (wrapped) and
            # the engine's pair force (none) in, forces, f out; the per-atom
            # array (peratom every step, the fix's default) leaves on its own
            # stream and is in place when end_of_step returns
            fix.post_force_host(xn, fn, arr, f_in=f0)
            # final_integrate: f in, the half kick, v out
            fix.final_integrate_host(fn, vn)
            # end_of_step: deposition and the grid
            fix.set_timestep(step_no[0])
            fix.end_of_step()

        for _ in range(2):
            host_step()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            host_step()
        torch.cuda.synchronize()
        t_e2e = ranks_reduce(time.perf_counter() - t0, "max", "cuda")
        # per atom: in x, v + x, f + f (5 x 24 B); out x, v + f + v (4 x 24 B) + the array (64 B)
        out.update(t_e2e=t_e2e, e2e_steps=e2e_steps, h2d=5 * 24 * n, d2h=4 * 24 * n + 64 * n)
    return out


def run_batched(args, dev):
    """The batched form: 64 independent cascades (32k-500k atoms, grids
    16^3-48^3) stepped together, one CUDA-graph launch per step, against the
    same replicas stepped one after another through the plain path."""
    import ephgb
    from ephgb import workloads as W

    with tempfile.TemporaryDirectory() as wd:
        bf = W.write_beta_file(os.path.join(wd, "synth.beta"))
        reps = W.batched_cascades(64, beta_file=bf)
        total = sum(at.n for _, at in reps)
        batch = ephgb.Batch(reps, dt=DT, device=dev)
        del reps
        batch.step(2)
        batch.synchronize()
        k = args.batch_steps
        t0 = time.perf_counter()
        batch.step(k)
        batch.synchronize()
        t_batch = time.perf_counter() - t0
        # the same replicas through the plain path, one after another
        t0 = time.perf_counter()
        for rep in batch.replicas:
            rep.step(k)
            rep.synchronize()
        t_seq = time.perf_counter() - t0
        return {"value": total * k / t_batch, "unit": METRIC, "replicas": len(batch.replicas), "atoms": total,
                "steps": k, "ms_per_step": 1000.0 * t_batch / k, "launches_per_step": batch.launches_per_step(),
                "sequential_value": total * k / t_seq, "speedup_vs_sequential": t_seq / t_batch,
                "timing": "host wall clock around the graph launches, synchronised"}


ADJ_CELLS, ADJ_GRID, ADJ_STEPS, ADJ_K, ADJ_DT = 20, (16, 16, 16), 200, 20, 0.001


def run_adjoint(args, dev, fd=True):
    """The adjoint workload: fcc Ni 20^3 cells (32,000 atoms), ions at 300 K,
    electrons at 2,000 K on a 16^3 grid, 200 steps of 1 fs, flags 7.  The beta
    file has 16 rho(r) knots and 64 beta(rho) knots.  Loss = sum_t (E[t] -
    E*[t])^2, E[t] the ion-to-electron energy of step t and E* the curve the
    plain method gives with a hidden beta(rho) (the start knots times
    1 + 0.3 sin(k/6)).  Gradient with respect to the 64 beta knots, the 16
    rho(r) knots, C_e and kappa_e, checkpoints every 20 steps; checked against
    central finite differences (h = 1e-6 relative) of the same forward.  Both
    passes and the plain method run as CUDA-graph replays.

    The beta table spans rho up to 1.26 (drho 0.02) so that no atom crosses
    the file's rho cutoff, where the reference sets beta = alpha = 0: such a
    crossing is a jump of the loss that no derivative describes.  The loss
    keeps smaller jumps (an atom crossing into another grid cell sees another
    T_e), and its rounding grows along the trajectory, so the finite
    differences have an error of their own: it is estimated by a second
    stencil, and the check is repeated with steps that balance rounding
    against those jumps."""
    import torch

    import ephgb
    from ephgb import workloads as W
    from ephgb.adjoint import Adjoint

    with tempfile.TemporaryDirectory() as wd:
        # beta(rho) with curvature over the table: the table construction's slope
        # weights are ill-conditioned where knots lie nearly on a line, and a
        # 1e-6 relative finite difference would measure that instead of the gradient
        bf = W.write_beta_file(os.path.join(wd, "adj.beta"), n_rho=16, n_beta=64, drho=0.02,
                               beta_fn=lambda r: 0.02 + 2.0 * r * r)
        nsteps = args.adjoint_steps
        atoms = W.fcc_lattice(ADJ_CELLS, seed=SEED + 7)
        words = W.fix_args(bf, seed=SEED, flags=7, T_e=2000.0, grid=ADJ_GRID)
        fix = ephgb.FixEPH(words, atoms, dt=ADJ_DT, mode=ephgb.MODE_FAST, device=dev)
        adj = Adjoint(fix, checkpoint_every=ADJ_K)
        r0, b0 = (c.copy() for c in adj.columns[0])
        hidden = b0 * (1.0 + 0.3 * np.sin(np.arange(b0.size) / 6.0))
        adj.set_knots(0, r0, hidden)
        target, _ = adj.forward(nsteps)
        adj.set_knots(0, r0, b0)

        def loss(r, b, C_e, kappa_e, steps=nsteps):
            adj.set_knots(0, r, b)
            adj.set_grid_constants(C_e, kappa_e)
            E, _ = adj.forward(steps)
            return float(((E - target[:steps]) ** 2).sum())

        c_cut = fix.counter("rho_cutoff")

        for _ in range(2):  # warm-up
            E, _ = adj.forward(nsteps)
            adj.backward(2.0 * (E - target), None)
        E, _ = adj.forward(nsteps)
        L0 = float(((E - target) ** 2).sum())
        adj.backward(2.0 * (E - target), None)
        t = adj.timing()
        g = adj.gradients(0)
        rho_cut_events = fix.counter("rho_cutoff") - c_cut
        # the plain method on the same system: eph_step, CUDA events on its stream
        plain = ephgb.FixEPH(words, atoms, dt=ADJ_DT, mode=ephgb.MODE_FAST, device=dev)
        stream = torch.cuda.Stream()  # a graph cannot be captured on the legacy default stream
        plain.set_stream(stream.cuda_stream)
        plain.set_graph(True)
        plain.step(10)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plain.step(nsteps)
        e1.record(stream)
        torch.cuda.synchronize()
        plain_ms = e0.elapsed_time(e1)
        # the same gradient with the whole trajectory recorded as one segment:
        # no recomputation (the recorded steps take ~4 GB at this size)
        fix1 = ephgb.FixEPH(words, atoms, dt=ADJ_DT, mode=ephgb.MODE_FAST, device=dev)
        adj1 = Adjoint(fix1, checkpoint_every=nsteps)
        adj1.set_knots(0, r0, b0)
        for _ in range(3):
            E1, _ = adj1.forward(nsteps)
            adj1.backward(2.0 * (E1 - target), None)
        t1 = adj1.timing()
        g1 = adj1.gradients(0)
        one_seg = {"backward_ms": t1["backward_ms"], "forward_ms": t1["forward_ms"],
                   "adjoint_over_forward": t1["backward_ms"] / t1["forward_ms"],
                   "gradient_identical_to_checkpointed": all(
                       np.array_equal(np.asarray(g[k]), np.asarray(g1[k])) for k in g)}
        del adj1, fix1
        res = {"workload": "fcc Ni 20^3 cells (32,000 atoms), ions 300 K, T_e 2,000 K, FDM 16^3, %d steps of 1 fs, "
                           "flags 7; 64 beta knots (beta = 0.02 + 2 rho^2), 16 rho(r) knots, C_e, kappa_e; "
                           "checkpoints every 20 steps" % nsteps,
               "loss": "sum_t (E[t] - E*[t])^2, E* from a hidden beta(rho)", "loss_value": L0,
               "forward_ms": t["forward_ms"], "backward_ms": t["backward_ms"], "plain_forward_ms": plain_ms,
               "adjoint_over_forward": t["backward_ms"] / t["forward_ms"],
               "forward_plus_adjoint_over_plain_forward": (t["forward_ms"] + t["backward_ms"]) / plain_ms,
               "forward_launches": t["forward_launches"], "backward_launches": t["backward_launches"],
               "rho_cutoff_crossings": rho_cut_events,
               "one_segment": one_seg,
               "timing": "CUDA events on the fix's stream (graph replays); backward includes the recomputation "
                         "from checkpoints"}
        if not fd:
            return res
        C0, K0 = adj.C_e, adj.kappa_e
        floor = np.abs(r0[r0 != 0]).min()  # a zero knot moves by 1e-6 of the smallest non-zero one

        def fd_grads(h, steps=nsteps, four_point=False, groups=("rho_knots", "beta_knots", "C_e", "kappa_e")):
            """Central differences (or the 4th-order 5-point stencil) of the loss
            over `steps` steps; h relative to each parameter, a number or a
            dict by parameter group."""
            hh = h if isinstance(h, dict) else {k: h for k in groups}

            def diff(f, d):
                if four_point:
                    return (8.0 * (f(1) - f(-1)) - (f(2) - f(-2))) / (12.0 * d)
                return (f(1) - f(-1)) / (2.0 * d)
            out = {}
            if "rho_knots" in groups:
                out["rho_knots"] = np.zeros(r0.size)
                for k in range(r0.size):
                    d = hh["rho_knots"] * max(abs(r0[k]), floor)
                    e_k = d * (np.arange(r0.size) == k)
                    out["rho_knots"][k] = diff(lambda s_: loss(r0 + s_ * e_k, b0, C0, K0, steps), d)
            if "beta_knots" in groups:
                out["beta_knots"] = np.zeros(b0.size)
                for k in range(b0.size):
                    d = hh["beta_knots"] * abs(b0[k])
                    e_k = d * (np.arange(b0.size) == k)
                    out["beta_knots"][k] = diff(lambda s_: loss(r0, b0 + s_ * e_k, C0, K0, steps), d)
            if "C_e" in groups:
                out["C_e"] = diff(lambda s_: loss(r0, b0, C0 * (1 + s_ * hh["C_e"]), K0, steps), hh["C_e"] * C0)
            if "kappa_e" in groups:
                out["kappa_e"] = diff(lambda s_: loss(r0, b0, C0, K0 * (1 + s_ * hh["kappa_e"]), steps),
                                      hh["kappa_e"] * K0)
            return out

        def rel_err(ga, fd):
            return {k: float(np.max(np.abs(np.asarray(ga[k]) - fd[k])) / np.abs(fd[k]).max()) for k in fd if k in ga}

        # The loss is only piecewise smooth (an atom crossing into another grid
        # cell sees another T_e), so every difference is taken at h and at h/2;
        # a parameter whose two differences disagree by more than 1e-6 of its
        # group's largest has a jump inside its stencil and is left out (and
        # counted).  The h/2 stencil also estimates the differences' own error.
        def checked(hs, groups=("rho_knots", "beta_knots", "C_e", "kappa_e")):
            f1 = fd_grads(hs, groups=groups)
            f2 = fd_grads({k: 0.5 * (hs[k] if isinstance(hs, dict) else hs) for k in groups}, groups=groups)
            errs, jumps, own = {}, {}, {}
            for k in groups:
                a1, a2, gk = np.atleast_1d(f1[k]), np.atleast_1d(f2[k]), np.atleast_1d(np.asarray(g[k]))
                scale = np.abs(a1).max()
                smooth = np.abs(a1 - a2) <= 1e-6 * scale
                jumps[k] = int((~smooth).sum())
                errs[k] = float(np.abs(gk - a1)[smooth].max() / scale) if smooth.any() else None
                own[k] = float(np.abs(a1 - a2)[smooth].max() / scale) if smooth.any() else None
            return errs, jumps, own

        # h = 1e-6 relative, as specified
        h = 1e-6
        err, jumps, fd_unc = checked(h)
        # steps that balance the loss's rounding (its error falls as 1/h) against
        # the jumps larger steps meet, for the two groups whose gradients are
        # small against the loss
        h_best = {"rho_knots": 3e-6, "beta_knots": 1e-6, "C_e": 1e-6, "kappa_e": 1e-4}
        err_b, jumps_b, _ = checked(h_best, groups=("rho_knots", "kappa_e"))
        err_b.update({k: err[k] for k in ("beta_knots", "C_e")})
        loss(r0, b0, C0, K0)
        def worst(e):
            return max(v for v in e.values() if v is not None)

        res.update({"grad_rel_err_vs_fd": err, "grad_rel_err_max": worst(err), "fd_h_relative": h,
                    "fd_params_with_a_jump": jumps, "fd_own_error_estimate": fd_unc,
                    "grad_rel_err_vs_fd_balanced_h": err_b, "balanced_h": h_best,
                    "fd_params_with_a_jump_balanced_h": jumps_b,
                    "grad_rel_err_max_balanced_h": worst(err_b),
                    "error_measure": "per parameter group max_k |g_k - fd_k| / max_k |fd_k| over the parameters "
                                     "whose differences at h and h/2 agree within 1e-6 (no jump of the loss "
                                     "inside the stencil)",
                    "params": int(r0.size + b0.size + 2)})
        return res


def run_adjoint_fit(args, dev):
    """Batched adjoint fitting (a reduced form of the 128-replica fitting
    workload; sizes in `config`): replicas of 16k-64k atoms (whole fcc cells),
    initial T_e uniform in 1,000-5,000 K, 16^3 grids, 1 fs steps; target mean-T_e
    curves made by the plain method with a hidden beta(rho) (64 knots, positive,
    smooth); Adam on the shared log(beta) knots from a flat guess, every
    iteration one batched forward and one batched backward graph."""
    import ephgb
    from ephgb import workloads as W
    from ephgb.adjoint import Adjoint, AdjointBatch, GRAD_BETA_KNOTS, fit_beta_batch

    R, nsteps, iters = args.fit_replicas, args.fit_steps, args.fit_iters
    rng = np.random.default_rng(SEED + 11)
    drho = 0.005
    kn = np.arange(64) * drho
    hidden = 0.02 + 2.0 * kn * kn + 0.01 * (1.0 + np.sin(kn / 0.03))
    with tempfile.TemporaryDirectory() as wd:
        bf = W.write_beta_file(os.path.join(wd, "fit.beta"), n_rho=16, n_beta=64, drho=drho,
                               beta_fn=lambda r: np.interp(r, kn, hidden))
        fixes, adjs, atoms_total = [], [], 0
        for r in range(R):
            cells = int(rng.integers(16, 26))  # 4 n^3 = 16,384 .. 62,500 atoms
            at = W.fcc_lattice(cells, seed=SEED + 100 + r)
            atoms_total += at.n
            words = W.fix_args(bf, seed=SEED + r, flags=7, T_e=float(rng.uniform(1000.0, 5000.0)), grid=(16, 16, 16))
            fix = ephgb.FixEPH(words, at, dt=ADJ_DT, mode=ephgb.MODE_FAST, device=dev)
            fixes.append(fix)
            adjs.append(Adjoint(fix, checkpoint_every=ADJ_K))
        batch = AdjointBatch(adjs)
        _, target = batch.forward(nsteps)
        beta0 = np.full(64, hidden.mean())
        # the knots the replicas' densities reach (non-zero gradient at the start)
        for a in adjs:
            a.set_knots(0, None, beta0)
        _, T = batch.forward(nsteps)
        batch.backward(None, T - target)
        g0 = sum(a.gradient(GRAD_BETA_KNOTS) for a in adjs)
        seen = np.abs(g0) > 1e-12 * np.abs(g0).max()
        # where the atoms' densities lie: weight of each knot interval
        rho = np.concatenate([f.get("rho") for f in fixes])
        hist_w = np.bincount(np.clip((rho / drho).astype(int), 0, 63), minlength=64).astype(float)
        hist_w /= hist_w.sum()
        t0 = time.perf_counter()

        def progress(it, loss):  # one line per Adam iteration on stderr (long runs)
            print(json.dumps({"fit_iteration": it, "loss": loss, "wall_s": time.perf_counter() - t0}),
                  file=sys.stderr, flush=True)

        beta, hist = fit_beta_batch(batch, nsteps, target, beta0, iters=iters, lr=0.05, log=progress)
        wall = time.perf_counter() - t0
        import torch
        free, total = torch.cuda.mem_get_info(dev)
        tb = batch.timing()
        # the same passes replica after replica (each its own graphs)
        for a in adjs:
            a.set_knots(0, None, beta)
        t1 = time.perf_counter()
        for a in adjs:
            E1, T1 = a.forward(nsteps)
            a.backward(None, T1 - target[adjs.index(a)])
        seq = time.perf_counter() - t1

        def err(b):
            return float(np.linalg.norm((b - hidden)[seen]) / np.linalg.norm(hidden[seen]))

        def werr(b):  # weighted by the share of atoms in each knot interval
            return float(np.sqrt((hist_w * (b - hidden) ** 2).sum() / (hist_w * hidden ** 2).sum()))

        # how strongly the data constrain each knot: its share of the loss
        # gradient's mass at the flat start (|dL/dbeta_k| / sum |dL/dbeta|)
        mass = np.abs(g0) / np.abs(g0).sum()
        order = np.argsort(-mass)
        top = order[:int(np.searchsorted(np.cumsum(mass[order]), 0.9)) + 1]  # knots holding 90 % of it

        def merr(b):
            return float(np.sqrt((mass * (b - hidden) ** 2).sum() / (mass * hidden ** 2).sum()))

        def top_err(b):
            return float(np.linalg.norm((b - hidden)[top]) / np.linalg.norm(hidden[top]))

        return {"workload": f"{R} replicas, {atoms_total:,} atoms in all (16k-64k each), T_e0 1,000-5,000 K, FDM 16^3, "
                            f"{nsteps} steps of 1 fs; 64 shared beta knots, Adam on log(beta), {iters} iterations, "
                            "flat initial guess",
                "loss_first": hist[0], "loss_last": hist[-1], "beta_rel_l2_err_initial": err(beta0),
                "beta_rel_l2_err_final": err(beta), "knots_constrained": int(seen.sum()),
                "beta_rel_err_density_weighted_initial": werr(beta0),
                "beta_rel_err_density_weighted_final": werr(beta),
                "knots_holding_atoms": int((hist_w > 0).sum()), "smoothness_weight": 10.0,
                "gradient_mass_per_knot": [round(float(m), 4) for m in mass],
                "knots_holding_90pct_of_gradient_mass": sorted(int(k) for k in top),
                "beta_rel_err_over_those_knots_initial": top_err(beta0),
                "beta_rel_err_over_those_knots_final": top_err(beta),
                "beta_rel_err_gradient_mass_weighted_initial": merr(beta0),
                "beta_rel_err_gradient_mass_weighted_final": merr(beta),
                "wall_s_per_iteration": wall / iters, "batched_forward_ms": tb["forward_ms"],
                "batched_backward_ms": tb["backward_ms"],
                "sequential_forward_plus_backward_s": seq,
                "batched_speedup_vs_sequential": seq / ((tb["forward_ms"] + tb["backward_ms"]) / 1000.0),
                "atom_steps_per_s_forward": atoms_total * nsteps / (tb["forward_ms"] / 1000.0),
                "device_memory_in_use_gb": (total - free) / 1e9}


# the reference decks' eam/alloy potential (Tests/MD_Run/Ni.eam: 10001-point
# tables, 6.5 A cut-off), kept xz-compressed with the test fixtures
REF_NI_EAM = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "ref_inputs",
                          "MD_Run_Ni.eam.xz")


def run_md_eam(args, dev):
    """Full MD: the bench workload with the engine's eam/alloy pair force on
    the reference decks' Ni.eam (Tests/MD_Run/run.lmp: pair_style eam/alloy)
    added to fix eph: atom-steps/s of the whole step and the pair force's
    share (phase timing)."""
    import lzma

    import torch

    import ephgb
    from ephgb import workloads as W

    with tempfile.TemporaryDirectory() as wd:
        words, atoms = make_system(wd)
        eam = os.path.join(wd, "Ni.eam")
        with open(REF_NI_EAM, "rb") as src, open(eam, "wb") as dst:
            dst.write(lzma.decompress(src.read()))
        fix = ephgb.FixEPH(words, atoms, dt=DT, mode=ephgb.MODE_FAST, device=dev, eam=(eam, ["Ni"]))
        stream = torch.cuda.Stream()
        fix.set_stream(stream.cuda_stream)
        fix.set_graph(True)
        fix.step(args.warmup)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        k = args.md_steps
        e0.record(stream)
        fix.step(k)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        fix.set_profiling(True)
        fix.step(10)
        fix.synchronize()
        ph = fix.phase_times()
        fix.set_profiling(False)
        total = sum(v[0] for v in ph.values())
        return {"workload": WORKLOAD + " + eam/alloy Ni.eam of the reference's MD_Run deck (6.5 A cut-off)",
                "atoms": atoms.n, "steps": k,
                "value": atoms.n * k / (ms / 1000.0), "unit": "MD atom-steps/s (pair force + fix eph)",
                "ms_per_step": ms / k, "pair_share": ph["pair"][0] / total,
                "phases_ms_per_step": {p: round(v[0] / 10, 4) for p, v in ph.items()},
                "pair_energy_per_atom": fix.pair_energy() / atoms.n}


def run_c1(args, dev, threads):
    """The reference's CPU-runnable case: fcc Ni 10^3 cells (4,000 atoms),
    300 K, dt 1 fs, 10^3 grid, flags 7 — 1,000 steps on the GPU (graph
    replay) against the CPU restatement on one host core and on all of them
    (a bounded sample of steps)."""
    import torch

    import ephgb
    from ephgb import workloads as W
    from oracle.bindings import OracleFix

    with tempfile.TemporaryDirectory() as wd:
        bf = W.write_beta_file(os.path.join(wd, "synth.beta"))
        at = W.fcc_lattice(10, seed=SEED)
        words = W.fix_args(bf, seed=SEED, flags=7, grid=(10, 10, 10))
        fix = ephgb.FixEPH(words, at, dt=0.001, device=dev)
        stream = torch.cuda.Stream()
        fix.set_stream(stream.cuda_stream)
        fix.set_graph(True)
        fix.step(20)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fix.step(1000)
        e1.record(stream)
        torch.cuda.synchronize()
        gpu = at.n * 1000 / (e0.elapsed_time(e1) / 1000.0)
        cpu = {}
        for th in (1, threads):
            ref = OracleFix(words, at, 0.001, threads=th)
            ref.step(None)
            t0 = ref.seconds(0)
            for _ in range(100):
                ref.step(None)
            cpu[th] = at.n * 100 / (ref.seconds(0) - t0)
        return {"workload": "fcc Ni 10^3 cells (4,000 atoms), 300 K, dt 1 fs, FDM 10^3, flags 7, model 4",
                "value": gpu, "unit": METRIC, "gpu_steps": 1000, "cpu_1_core": cpu[1], "cpu_all_cores": cpu[threads],
                "cores": threads, "cpu_sample": "100 steps, fix hooks only", "speedup_vs_all_cores": gpu / cpu[threads],
                "ms_per_step": at.n / gpu * 1000.0}


def cpu_baseline(threads, steps=1, warm=1):
    """The CPU restatement (oracle port) on the same workload: `steps` steps
    of the full system after `warm` warm-up steps; time of the fix's own hooks
    (integrator, post_force, end_of_step), neighbour builds excluded as in
    LAMMPS's Modify timer."""
    from oracle.bindings import OracleFix

    with tempfile.TemporaryDirectory() as wd:
        words, atoms = make_system(wd)
        fix = OracleFix(words, atoms, DT, threads=threads)
        for _ in range(warm):
            fix.step(None)
        t0 = fix.seconds(0)
        for _ in range(steps):
            fix.step(None)
        t = fix.seconds(0) - t0
        return {"value": atoms.n * steps / t, "unit": METRIC, "cores": threads, "kind": "port",
                "sample": f"{steps} step(s) of the full {atoms.n}-atom workload after {warm} warm-up step(s); "
                          f"fix hooks only (neighbour builds excluded), OpenMP over atoms, {threads} threads",
                "seconds": t}


def main():
    global CELLS, GRID, WORKLOAD
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true", help="omit the cpu_baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="omit the end-to-end leg")
    ap.add_argument("--no-fp64-pairs", action="store_true", help="omit the leg with FP64 pair terms")
    ap.add_argument("--no-batched", action="store_true", help="omit the batched-replicas leg")
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--no-adjoint", action="store_true", help="omit the adjoint leg")
    ap.add_argument("--only-adjoint", action="store_true", help="run the adjoint leg alone (profiling)")
    ap.add_argument("--adjoint-steps", type=int, default=ADJ_STEPS)
    ap.add_argument("--no-adjoint-fd", action="store_true", help="skip the finite-difference check")
    ap.add_argument("--no-fit", action="store_true", help="omit the batched adjoint fitting leg")
    ap.add_argument("--no-md", action="store_true", help="omit the full-MD (EAM pair force) leg")
    ap.add_argument("--no-c1", action="store_true", help="omit the 4,000-atom CPU-runnable case")
    ap.add_argument("--only-md", action="store_true", help="run the full-MD leg alone")
    ap.add_argument("--md-steps", type=int, default=50)
    ap.add_argument("--only-fit", action="store_true", help="run the batched adjoint fitting leg alone")
    ap.add_argument("--fit-replicas", type=int, default=16)
    ap.add_argument("--fit-steps", type=int, default=100)
    ap.add_argument("--fit-iters", type=int, default=60)
    ap.add_argument("--cells", type=int, default=CELLS, help="fcc cells per edge (profiling cases)")
    ap.add_argument("--grid", type=int, default=GRID[0], help="FDM cells per edge (profiling cases)")
    ap.add_argument("--autotune-skin", action="store_true",
                    help="choose the list skin by eph_autotune_list_skin before the timed steps")
    ap.add_argument("--autotune-steps", type=int, default=40, help="steps per trial window of --autotune-skin")
    ap.add_argument("--list-skin", type=float, default=None,
                    help="skin of the kept candidate lists in A (0: bin search every step; default: the library's)")
    args = ap.parse_args()
    if args.cells != CELLS or args.grid != GRID[0]:
        CELLS, GRID = args.cells, (args.grid,) * 3
        WORKLOAD = (f"fcc Ni {CELLS}^3 cells ({4 * CELLS ** 3:,} atoms), 10 keV PKA, dt 0.5 fs, FDM {GRID[0]}^3, "
                    "flags 7, model 4")
    args.warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    threads = os.cpu_count() or 1

    if args.impl == "reference":
        # the reference algorithm on the host cores (the oracle port: the
        # reference's own sources need its engine and are not on this host)
        if rank != 0:
            return
        k = max(1, min(args.steps, 3))
        cb = cpu_baseline(threads, steps=k, warm=1)
        line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": METRIC, "n_gpus": 0,
                "steps": k, "warmup": 1, "ms_per_step": 1000.0 * cb["seconds"] / k, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "steps_timed": k},
                "cpu_baseline": {k2: cb[k2] for k2 in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": cb["value"], "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch

    if args.only_md:
        print(json.dumps(run_md_eam(args, int(os.environ.get("LOCAL_RANK", rank)))))
        return
    if args.only_fit:
        print(json.dumps(run_adjoint_fit(args, int(os.environ.get("LOCAL_RANK", rank)))))
        return
    if args.only_adjoint:
        print(json.dumps(run_adjoint(args, int(os.environ.get("LOCAL_RANK", rank)), fd=not args.no_adjoint_fd)))
        return
    if world > 1:
        torch.distributed.init_process_group("nccl")
    res = run_gpu(args, rank, world)
    n = res["n"]
    value = job_value(world, n, args.steps, res["ms"])
    hbm, peak_src = peaks()

    def roofline(phase, kernel, nbytes, dram_ratio, pipes):
        ms_p, nl_p = res["phases"][phase]
        t_launch = ms_p / max(nl_p, 1) / 1000.0
        achieved = nbytes / t_launch / 1e9
        return {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_source": peak_src, "traffic": dram_ratio * nbytes,
                "algorithmic_bytes": nbytes, "launch_ms": t_launch * 1000.0, "pipes_ncu_131k": pipes,
                "note": "df64 pair arithmetic on the FP32 pipe; latency-bound on the neighbours' records "
                        "(ncu: long-scoreboard stalls first)"}
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["ms"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (pair terms df64)", "data": "synthetic",
        "config": {"workload": WORKLOAD, "atoms_per_gpu": n, "grid": list(GRID), "dt_ps": DT,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (pair cache ~%d MB)" % (res["n_pairs"] * 52 // 2 ** 20),
                   "mode": "fast", "pair_arithmetic": "df64", "xi": "device Philox4x32-10"},
        "gpu_launches": res["launches"],
        "roofline": roofline("density", "k_density_list_df", density_bytes(n, res["n_pairs"]),
                             DENSITY_DRAM_OVER_ALGORITHMIC, DENSITY_PIPES),
        "roofline_forces": roofline("forces", "k_forces_df", forces_bytes(n, res["n_pairs"]),
                                    FORCES_DRAM_OVER_ALGORITHMIC, FORCES_PIPES),
        # the whole step against HBM with the scope's own byte count per atom-step
        "roofline_step": {"bound": "hbm", "bytes_per_atom_step": step_bytes_8d(),
                          "achieved": step_bytes_8d() * n / (res["ms"] / args.steps / 1000.0) / 1e9,
                          "peak": hbm, "unit": "GB/s",
                          "frac": step_bytes_8d() * n / (res["ms"] / args.steps / 1000.0) / 1e9 / hbm,
                          "note": "4 n_L P + 156 + 224 B per atom-step, n_L = 78, P = 3; the sweeps are bound "
                                  "by issue and latency, not by these bytes"},
        "phases_ms": {k: round(v[0], 3) for k, v in res["phases"].items()},
        "clocks": res["clocks"],
        "pairs_per_atom": res["n_pairs"] / n,
        "wraps": res["rebuilds"],
        "list_skin_A": res["list_skin"][0] if res["list_skin"][1] else 0.0,
        "list_builds": res["list_builds"],  # in the timed steps
    }
    if "ms64" in res:
        line["fp64_pairs"] = {"value": job_value(world, n, res["steps64"], res["ms64"]), "unit": METRIC,
                              "ms_per_step": res["ms64"] / res["steps64"], "steps": res["steps64"],
                              "note": "the same workload with the pair terms in FP64 (EPH_PAIRS_FP64), "
                                      "timed after the main steps from the state they reached"}
    if res.get("skin_autotuned") is not None:
        line["list_skin_autotuned"] = {"candidates_A": list(SKIN_CANDIDATES), "chosen_A": res["skin_autotuned"],
                                       "window_steps": args.autotune_steps}
    if "t_e2e" in res:
        line["e2e"] = {"value": world * n * res["e2e_steps"] / res["t_e2e"], "unit": METRIC,
                       "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"], "steps": res["e2e_steps"],
                       "sequence": "the hooks and copies of the LAMMPS fix eph/gb (fix_eph_gb.cpp) with its default "
                                   "settings on a re-neighbouring step without re-sorting, pinned host arrays",
                       "timing": "host wall clock, synchronised"}
    if not args.no_batched:
        line["batched"] = run_batched(args, int(os.environ.get("LOCAL_RANK", rank)))
        line["batched"]["value"] = ranks_reduce(line["batched"]["value"], "sum", "cuda")
    if rank == 0 and not args.no_adjoint:
        line["adjoint"] = run_adjoint(args, int(os.environ.get("LOCAL_RANK", rank)), fd=not args.no_adjoint_fd)
    if rank == 0 and not args.no_c1:
        line["c1"] = run_c1(args, int(os.environ.get("LOCAL_RANK", rank)), threads)
    if rank == 0 and not args.no_md:
        line["md_eam"] = run_md_eam(args, int(os.environ.get("LOCAL_RANK", rank)))
    if rank == 0 and not args.no_fit:
        line["adjoint_fit"] = run_adjoint_fit(args, int(os.environ.get("LOCAL_RANK", rank)))
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = {k: v for k, v in cpu_baseline(threads, steps=1, warm=1).items() if k != "seconds"}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
