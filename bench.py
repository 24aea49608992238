"""Benchmark: NNP energy+force atom-evaluations per second on one GB300 (and N replicas).

Workload: 256 binary A/B structures, N ~ U{32..512} atoms each (74,710 atoms), number density
0.05 /A^3, rc = 6.5 A, 72 symmetry functions per atom (12 radial per species + 16 angular per
species pair), 72-64-64-1 softplus networks; one packed batch per step (neighbour list,
symmetry functions, networks, forces, virials, per-structure energies).

  value  : atom-evaluations/s with the batch resident in HBM (device-timed with CUDA events on
           the library's stream, L2 flushed by a 256 MiB write between steps, outside the timed
           events), mixed precision (FP32 geometry/basis/forces, BF16 hi/lo tensor-core networks
           with FP32 accumulation, FP64 sums).
  e2e    : the same through ann_compute with the batch in page-locked host memory (H2D of
           positions/types/cells/offsets and D2H of energies/forces/virials inside the timed
           region, every step), wall-clock.
  fp64   : the plain FP64 GPU form on the same batch (the 5x target's denominator).
  --impl reference : the CPU path (the FP64 oracle that restates the reference's code) on all host
           cores, on a bounded sample of the same workload.
  training : structures/s of one training step (loss, adjoint, parameter gradient) on the
           64-structure batch with LJ labels, mixed and FP64 (secondary keys).
  md     : atom-steps/s and energy drift of velocity-Verlet MD on the 262,144-atom FCC Ar box.
  parity / accuracy : the FP64 oracle on the whole batch against the FP64 GPU form (relative
           errors) and the mixed form (meV/atom, meV/A).
  precision_study / small_box / lammps / network_forms : the 32,000-atom ternary box (96-128-128-1),
           the 108-atom argon box, the caller-list path and the three tensor-core operand forms.
Multi-GPU: structures are independent, so each rank runs its own full batch (weak scaling);
no collective on the data path, a barrier and a max over ranks around the timed region.
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
sys.path.insert(0, str(ROOT))

METRIC = "NNP E+F atom-evals/s: batched BF16/FP32 vs plain FP64 on GB300 at <=10 meV/A force err"
WORKLOAD = ("256 binary A/B structures, N~U{32..512} (seeded), rho=0.05/A^3, 1.8 A min distance, rc=6.5 A, "
            "72 symmetry functions (12 radial/species + 16 angular/pair), 72-64-64-1 softplus nets, one packed batch")


def _env_rank():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        rows = [r for r in self.rows if len(r) >= 9]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def algorithmic_work(ctx, offs, posn, types, cell):
    """Exact pair / triplet counts of the batch (within rc, per type block) from an FP64 pass, and the
    algorithmic work of the force kernel by the counting conventions: per pair 15 flop + cos/sin
    pair, radial function F = 8 flop + 1 exp; per triplet 20 flop + 1 exp per damping group,
    angular function F = 10 flop + 1 pow (2 MUFU). Bytes: neighbour row (16 B geometry + 4 B index
    read, 12 B Newton-3rd write) per pair, dE/dG row and 48 B force/virial per atom."""
    from ann_gb300 import FP64
    ctx.compute(offs, posn, types, cell, precision=FP64)
    i, j, img, r = ctx.neighbors(with_vectors=True)
    d = np.linalg.norm(r, axis=1)
    keep = d < ctx.rc
    i, j = i[keep], j[keep]
    T = ctx.ntypes
    N = len(types)
    cnt = np.zeros((N, T), np.int64)
    np.add.at(cnt, (i, types[j]), 1)
    nR = {}
    nA = {}
    ng = 2  # angular damping groups of this potential (eta_B in {0.003, 0.01})
    nin = {t: ctx.num_inputs(t) for t in range(T)}
    # the workload's potential has the same basis sizes for every block
    nr_block = 12
    na_block = 16
    pairs = cnt.sum()
    trip = 0
    for a in range(T):
        for b in range(a, T):
            if a == b:
                trip += int((cnt[:, a] * (cnt[:, a] - 1) // 2).sum())
            else:
                trip += int((cnt[:, a] * cnt[:, b]).sum())
    flops = pairs * (15 + 8 * nr_block) + trip * (20 + 10 * na_block)
    mufu = pairs * (2 + nr_block) + trip * (2 * na_block + ng)
    imax = max(nin.values())
    bytes_ = pairs * (16 + 4 + 12) + N * (imax * 4 + 48)
    return dict(pairs=int(pairs), triplets=int(trip), natoms=N, force_flops=float(flops), force_mufu=float(mufu),
                force_bytes=float(bytes_), symm_flops=float(pairs * (15 + 6 * nr_block) + trip * (20 + 4 * na_block)),
                symm_mufu=float(pairs * (2 + nr_block) + trip * (2 * na_block + ng)))


def cpu_reference(offs, posn, types, cell, pot_text, budget_s=12.0, steps=1, warmup=0, threads=None):
    """The oracle (CPU restatement of the reference's path, FP64) on all host cores over a bounded
    sample of the workload's structures; returns atom-evals/s and the sample description."""
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_lib import Oracle
    orc = Oracle(timed=True)
    pot = orc.load_text(pot_text)
    threads = threads or os.cpu_count() or 1
    S = len(offs) - 1

    def run(k):
        o = offs[: k + 1]
        n = int(o[-1])
        t0 = time.perf_counter()
        pot.compute(o, posn[:n], types[:n], cell[:k], forces=True, nthreads=threads)
        return time.perf_counter() - t0, n

    # size the sample: time a first chunk of `threads` structures, then scale to the budget
    k = min(S, threads)
    dt, n = run(k)
    per_struct = dt / max(k, 1) * threads
    k = int(min(S, max(threads, budget_s / max(per_struct, 1e-6) * threads / 1.0)))
    k = max(1, min(S, (k // threads) * threads or k))
    for _ in range(warmup):
        run(k)
    rates = []
    for _ in range(max(1, steps)):
        dt, n = run(k)
        rates.append(n / dt)
    return dict(value=float(np.median(rates)), unit="atom-evals/s", cores=threads, kind="port",
                sample=f"first {k} of {S} structures ({n} atoms) of the workload, FP64 oracle, {threads} threads, "
                       f"structures block-distributed over threads (thread::Dist rule)")


def oracle_parity(offs, posn, types, cell, pot_text, E64, F64, W64, Emx, Fmx, Wmx, threads=None):
    """The FP64 oracle (accurate build, no FP contraction) on the whole batch, all host cores: the
    FP64 GPU form's largest relative errors (bars: 1e-10) and the mixed form's errors in meV/atom
    and meV/A (bars: 1 and 10), both against the oracle."""
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_lib import Oracle
    pot = Oracle().load_text(pot_text)
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    Eo, Fo, Wo, _, _ = pot.compute(offs, posn, types, cell, forces=True, nthreads=threads)
    dt = time.perf_counter() - t0

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))

    nat = np.diff(offs)
    fp64 = {"e_rel_max": rel(E64, Eo), "f_rel_max": rel(F64, Fo), "w_rel_max": rel(W64, Wo), "bar": 1e-10}
    fp64["within_bar"] = bool(max(fp64["e_rel_max"], fp64["f_rel_max"], fp64["w_rel_max"]) < 1e-10)
    mixed = {"e_mev_atom_max": float(np.max(np.abs(Emx - Eo) / nat) * 1e3),
             "f_mev_A_max": float(np.max(np.abs(Fmx - Fo)) * 1e3),
             "f_mev_A_rms": float(np.sqrt(np.mean((Fmx - Fo) ** 2)) * 1e3),
             "w_rel_max": rel(Wmx, Wo), "bars": "1 meV/atom, 10 meV/A"}
    mixed["within_bar"] = bool(mixed["e_mev_atom_max"] < 1.0 and mixed["f_mev_A_max"] < 10.0)
    return {"reference": f"FP64 oracle (CPU restatement of the reference path) on all {len(nat)} structures "
                         f"({int(offs[-1])} atoms), {threads} threads, {dt:.1f} s",
            "fp64_gpu_vs_oracle": fp64, "mixed_vs_oracle": mixed}, Eo, Fo


def resident_timer(ctx, dev):
    """CUDA-event times (ms) of E+F evaluations of a batch resident in HBM, on the library's stream,
    with the L2 cache flushed by a 256 MiB write between steps, outside the timed events."""
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")

    def run(offs, posn, types, cell, prec, steps, warm):
        ctx.upload(offs, posn, types, cell)
        for _ in range(warm):
            ctx.compute_resident(prec)
        ctx.download(forces=False, virial=False)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        torch.cuda.synchronize(dev)
        for k in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                ev[k][0].record(stream)
            ctx.compute_resident(prec)
            ev[k][1].record(stream)
        ctx.download(forces=False, virial=False)
        torch.cuda.synchronize(dev)
        return [a.elapsed_time(b) for a, b in ev]

    def phases(offs, posn, types, cell, prec, steps, warm):
        ctx.profile_phases(True)
        ctx.upload(offs, posn, types, cell)
        out = []
        for k in range(warm + steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            ctx.compute_resident(prec)
            ctx.synchronize()
            if k >= warm:
                out.append(ctx.phase_times())
        ctx.profile_phases(False)
        return dict(zip(PHASES, map(float, np.mean(np.array(out), axis=0))))

    run.phases = phases
    return run


PHASES = ["neighbour_list", "type_lists", "symmetry_functions", "networks", "forces", "reductions"]


def _errors_vs(E, F, Eo, Fo, offs):
    nat = np.diff(offs)
    return {"e_mev_atom_max": float(np.max(np.abs(E - Eo) / nat) * 1e3), "f_mev_A_max": float(np.max(np.abs(F - Fo)) * 1e3),
            "f_mev_A_rms": float(np.sqrt(np.mean((F - Fo) ** 2)) * 1e3)}


def network_forms_leg(dev, offs, posn, types, cell, pot_text, Eo, Fo, steps=10, warmup=3):
    """The E+F workload with each operand form of the tensor-core networks (1: BF16 activations and
    weights; 2: activations split hi + lo; 3: both split), FP32 accumulation throughout: step time
    and network-phase time (CUDA events) and the errors against the FP64 oracle."""
    from ann_gb300 import MIXED, Context
    out = {"workload": "the E+F workload above", "reference": "FP64 oracle on the whole batch"}
    N = int(offs[-1])
    for split in (1, 2, 3):
        ctx = Context(device=dev, mlp_backend=2, tc_split=split)
        try:
            ctx.load_text(pot_text)
            E, F, _ = ctx.compute(offs, posn, types, cell, precision=MIXED)
            run = resident_timer(ctx, dev)
            ms = float(np.mean(run(offs, posn, types, cell, MIXED, steps, warmup)))
            ph = run.phases(offs, posn, types, cell, MIXED, steps, warmup)
            out[f"split{split}"] = dict(_errors_vs(E, F, Eo, Fo, offs), ms_per_step=ms, atom_evals_per_s=N / (ms * 1e-3),
                                        networks_ms=ph["networks"], forms=[ctx.network_form(t) for t in range(ctx.ntypes)])
        finally:
            ctx.close()
    return out


def precision_study_leg(dev, steps=10, warmup=3):
    """The large-frame precision study: one ternary A:B:C = 1:1:2 periodic box of 32,000 atoms (jittered
    simple-cubic lattice 40 x 40 x 20 at 0.07 /A^3, sigma 0.15 A), rc = 6 A, 96 inputs (16 radial per
    species, 8 angular per pair), 96-128-128-1 tanh networks. The FP64 oracle (atoms split over all
    host cores) against the FP64 GPU form (relative errors) and against each mixed form (meV/atom,
    meV/A), with their E+F throughput (CUDA events, box resident, L2 flushed between steps)."""
    import tempfile
    from ann_gb300 import FP64, MIXED, Context
    from ann_gb300 import workloads as WL
    from ann_gb300.api import pack_batch
    structs = WL.config4()
    offs, posn, types, cell = pack_batch(structs)
    N = int(offs[-1])
    ctx = Context(device=dev)
    WL.make_potential(ctx, 4)
    WL.precondition(ctx, offs, posn, types, cell)
    with tempfile.TemporaryDirectory() as td:
        p = Path(td) / "pot.ann"
        ctx.write(p)
        pot_text = p.read_text()
    ctx.close()
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_lib import Oracle
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    Eo, Fo, Wo, _, _ = Oracle().load_text(pot_text).compute(offs, posn, types, cell, nthreads=threads)
    t_orc = time.perf_counter() - t0
    out = {"workload": f"ternary box, {N} atoms (1:1:2), rho 0.07/A^3, rc 6 A, 96 inputs, 96-128-128-1 tanh",
           "reference": f"FP64 oracle, atoms split over {threads} threads, {t_orc:.1f} s"}
    forms = (("fp64", FP64, {}), ("mixed_tc_split3", MIXED, {"mlp_backend": 2, "tc_split": 3}),
             ("mixed_tc_split2", MIXED, {"mlp_backend": 2, "tc_split": 2}),
             ("mixed_tc_split1", MIXED, {"mlp_backend": 2, "tc_split": 1}), ("mixed_simt", MIXED, {"mlp_backend": 1}))
    for name, prec, kw in forms:
        ctx = Context(device=dev, **kw)
        try:
            ctx.load_text(pot_text)
            E, F, Wv = ctx.compute(offs, posn, types, cell, precision=prec)
            run = resident_timer(ctx, dev)
            ms = float(np.mean(run(offs, posn, types, cell, prec, steps, warmup)))
            ph = run.phases(offs, posn, types, cell, prec, steps, warmup)
            r = dict(_errors_vs(E, F, Eo, Fo, offs), ms_per_step=ms, atom_evals_per_s=N / (ms * 1e-3), phase_ms=ph)
            if prec == FP64:
                r["e_rel"] = float(abs(E[0] - Eo[0]) / abs(Eo[0]))
                r["f_rel_max"] = float(np.max(np.abs(F - Fo)) / np.max(np.abs(Fo)))
                r["w_rel_max"] = float(np.max(np.abs(Wv - Wo)) / np.max(np.abs(Wo)))
            else:
                r["forms"] = [ctx.network_form(t) for t in range(ctx.ntypes)]
            out[name] = r
        finally:
            ctx.close()
    return out


def small_box_leg(dev, steps=200, warmup=20):
    """The 108-atom FCC argon box (3 x 3 x 3 cells, a = 5.26 A, 0.1 A jitter), 16 inputs, 16-20-20-1
    tanh: the FP64 GPU form against the FP64 oracle (relative errors), the mixed form against the
    oracle (meV/atom, meV/A), E+F throughput of both forms with the box resident (CUDA events, one
    launch sequence per step: this size is launch-bound) and of the oracle on one host thread."""
    import tempfile
    from ann_gb300 import FP64, MIXED, Context
    from ann_gb300 import workloads as WL
    from ann_gb300.api import pack_batch
    structs = WL.config1()
    offs, posn, types, cell = pack_batch(structs)
    N = int(offs[-1])
    ctx = Context(device=dev, use_graphs=True)
    try:
        WL.make_potential(ctx, 1)
        with tempfile.TemporaryDirectory() as td:
            p = Path(td) / "pot.ann"
            ctx.write(p)
            pot_text = p.read_text()
        ctx.load_text(pot_text)
        sys.path.insert(0, str(ROOT / "tests"))
        from oracle_lib import Oracle
        orc = Oracle(timed=True).load_text(pot_text)
        Eo, Fo, Wo, _, _ = Oracle().load_text(pot_text).compute(offs, posn, types, cell, nthreads=1)
        reps, t0 = 0, time.perf_counter()
        while reps < 3 or time.perf_counter() - t0 < 2.0:
            orc.compute(offs, posn, types, cell, nthreads=1)
            reps += 1
        cpu = N * reps / (time.perf_counter() - t0)
        out = {"workload": f"FCC Ar {N} atoms, rc 6 A, 16 inputs, 16-20-20-1 tanh",
               "cpu_oracle_1_thread": cpu, "unit": "atom-evals/s"}
        run = resident_timer(ctx, dev)
        for name, prec in (("fp64", FP64), ("mixed", MIXED)):
            E, F, Wv = ctx.compute(offs, posn, types, cell, precision=prec)
            ms = float(np.median(run(offs, posn, types, cell, prec, steps, warmup)))
            r = dict(_errors_vs(E, F, Eo, Fo, offs), ms_per_step=ms, atom_evals_per_s=N / (ms * 1e-3))
            if prec == FP64:
                r["e_rel"] = float(abs(E[0] - Eo[0]) / abs(Eo[0]))
                r["f_rel_max"] = float(np.max(np.abs(F - Fo)) / np.max(np.abs(Fo)))
                r["w_rel_max"] = float(np.max(np.abs(Wv - Wo)) / np.max(np.abs(Wo)))
            out[name] = r
    finally:
        ctx.close()
    return out


def training_leg(dev, steps=10, warmup=3):
    """Training throughput on the 64-structure binary batch with Lennard-Jones labels: one
    ann_train_forward + ann_train_backward (loss, adjoint, parameter gradient) + ann_adam_step
    (optimiser step on the resident parameters) per step: host arrays and labels in, the loss out,
    the gradient kept on the device for the optimiser; wall-clock per step. The staged form is the
    reference trainer's loop (neighbour lists and symmetry functions of the training set built once,
    nnptefr2.cpp:2690-2703): ann_train_forward_staged in place of ann_train_forward."""
    from ann_gb300 import FP64, MIXED, Context
    from ann_gb300 import workloads as WL
    from ann_gb300.api import pack_batch
    structs = WL.config3()
    offs, posn, types, cell = pack_batch(structs)
    Eref, Fref = WL.lennard_jones(structs)
    Fref = np.concatenate(Fref)
    ctx = Context(device=dev)
    WL.make_potential(ctx, 3)
    WL.precondition(ctx, offs, posn, types, cell)
    out = {"workload": f"{len(structs)} binary structures, N~U{{32..256}} ({int(offs[-1])} atoms), LJ labels, "
                       "loss = mean (dE/N)^2 + 0.1 mean |dF|^2/3, Adam step on the device",
           "unit": "structures/s", "nparams": int(ctx.nparams)}
    p0 = ctx.get_params()
    # "<prec>": every step sends the batch and its labels and builds lists and symmetry functions;
    # "<prec>_staged": the reference trainer's loop, lists and symmetry functions built once for the
    # training set (before the timed steps), each step networks + forces + loss + adjoint + gradient
    # + optimiser step (ann_train_forward_staged)
    for name, prec, staged in (("mixed", MIXED, False), ("mixed_staged", MIXED, True), ("fp64", FP64, False),
                               ("fp64_staged", FP64, True)):
        ctx.set_params(p0)
        ctx.adam_init(1e-4, 0.9, 0.999, 1e-16)

        def fwd(first):
            if staged and not first:
                return ctx.train_forward_staged(1.0, 0.1, precision=prec)
            return ctx.train_forward(offs, posn, types, cell, Eref, Fref, 1.0, 0.1, precision=prec)

        for k in range(warmup):
            fwd(k == 0)
            ctx.train_backward(download=False)
            ctx.adam_step()
        t0 = time.perf_counter()
        for _ in range(steps):
            loss = fwd(False)
            ctx.train_backward(download=False)
            ctx.adam_step()
        ctx.synchronize()
        dt = (time.perf_counter() - t0) / steps
        out[name] = len(structs) / dt
        out[name + "_ms_per_step"] = dt * 1e3
        out[name + "_loss"] = float(loss[0])
    ctx.close()
    return out


def md_leg(dev, steps=1000, warmup=20):
    """Velocity-Verlet MD of the 262,144-atom FCC argon box (16-32-32-1 tanh networks whose weights
    hold a Lennard-Jones argon pair potential, workloads.lj_argon_text; dt = 2 fs, list cutoff
    rc + 0.5 A, rebuild at 0.25 A displacement), mixed precision: atom-steps/s, the total-energy
    drift and the final temperature. The crystal stays a crystal, so the per-step cost is that of
    a fixed neighbour count (randomly initialised weights attract atoms without bound: the box
    collapses, heats to thousands of kelvin and the triplet count triples within 2 ps)."""
    from ann_gb300 import MIXED, Context
    from ann_gb300 import workloads as WL
    x, v, t, R = WL.config5()
    ctx = Context(device=dev)
    ctx.load_text(WL.lj_argon_text(5))
    ctx.md_init(x, v, t, R, np.array([WL.MASS["Ar"]]), dt_fs=2.0, skin=0.5, precision=MIXED)
    ctx.md_run(warmup)
    pe0, ke0, _ = ctx.md_run(1)
    t0 = time.perf_counter()
    pe, ke, rebuilds = ctx.md_run(steps)
    dt = time.perf_counter() - t0
    n = len(t)
    ps = steps * 2.0e-3
    ctx.close()
    return {"workload": f"FCC Ar {n} atoms, 80 K, dt 2 fs, {steps} steps", "atom_steps_per_s": n * steps / dt,
            "ms_per_step": dt / steps * 1e3, "rebuilds": int(rebuilds),
            "drift_mev_atom_ps": float((pe + ke - pe0 - ke0) / n * 1e3 / ps),
            "T_end_K": float(2.0 * ke / (3.0 * n * 8.617333262e-5)), "precision": "mixed"}


def lammps_leg(dev, steps=20, warmup=3, skin=2.0):
    """The LAMMPS pair-style path (ann_compute_list) on the 262,144-atom FCC argon box (16-32-32-1
    tanh networks holding the Lennard-Jones argon potential, mixed precision) as one MD domain:
    local atoms plus ghosts within rc + skin (LAMMPS's default metal-units skin, 2 A), a full list
    of the same radius. Times, end to end from host arrays to host forces of all local and ghost
    atoms: a reneighbouring step (list, types and positions sent) and a step between
    reneighbourings (ANN_LIST_KEEP: positions only)."""
    from ann_gb300 import MIXED, Context
    from ann_gb300 import workloads as WL
    x, _, t, R = WL.config5()
    ctx = Context(device=dev)
    ctx.load_text(WL.lj_argon_text(5))
    X, T, owner, nn, nb = WL.ghost_domain(x, t, R, ctx.rc + skin)
    n, nall = len(t), len(X)

    def run(keep, k):
        ts = []
        for _ in range(k):
            t0 = time.perf_counter()
            if keep:
                E, F, _, _ = ctx.compute_list(X, None, None, None, precision=MIXED, keep=True, inum=n, virial=False)
            else:
                E, F, _, _ = ctx.compute_list(X, T, nn, nb, precision=MIXED, virial=False)
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts)), E, F

    run(False, warmup)
    t_full, E, F = run(False, steps)
    run(True, warmup)
    t_keep, E2, _ = run(True, steps)
    folded = np.zeros((n, 3))
    np.add.at(folded, owner, F)
    ctx.close()
    h2d_full = X.nbytes + T.nbytes + nn.nbytes + nb.nbytes + 8 * (n + 1)
    return {"workload": f"FCC Ar {n} local + {nall - n} ghost atoms, full list rc + {skin} A ({len(nb) / n:.1f} entries per atom)",
            "precision": "mixed", "reneighbour_step_ms": t_full * 1e3, "keep_step_ms": t_keep * 1e3,
            "atom_evals_per_s_keep": n / t_keep, "atom_evals_per_s_reneighbour": n / t_full,
            "h2d_bytes_reneighbour": int(h2d_full), "h2d_bytes_keep": int(X.nbytes), "d2h_bytes": int(24 * nall + 8),
            "energy_equal_keep_vs_full": bool(E == E2), "net_force_after_fold": float(np.abs(folded.sum(axis=0)).max())}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the FP64 oracle run over the whole batch (accuracy and parity)")
    ap.add_argument("--nstruc", type=int, default=256)
    ap.add_argument("--no-extras", action="store_true", help="skip the training and MD legs")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the built-in launch shapes (no autotuner launches before the timed steps, e.g. for "
                         "ncu captures that select launches by position)")
    ap.add_argument("--only", choices=["training", "md", "lammps", "precision", "small"],
                    help="run one secondary leg alone with --steps / --warmup and print its JSON (for profiling)")
    args = ap.parse_args()
    rank, world, local = _env_rank()
    W_ = max(args.warmup, 3)
    if args.only:
        leg = {"training": training_leg, "md": md_leg, "lammps": lammps_leg, "precision": precision_study_leg,
               "small": small_box_leg}[args.only]
        print(json.dumps({args.only: leg(local if world > 1 else 0, steps=args.steps, warmup=args.warmup)}))
        return

    from ann_gb300 import workloads as WL
    from ann_gb300.api import pack_batch

    structs = WL.config2(nstruc=args.nstruc)
    offs, posn, types, cell = pack_batch(structs)
    N = int(offs[-1])

    if args.impl == "reference":
        if world > 1 and rank != 0:
            return
        # same basis and networks as the GPU arm (host-only construction; the input scaling does
        # not change the CPU cost)
        pot_text = WL.config_potential_text(2)
        cb = cpu_reference(offs, posn, types, cell, pot_text, steps=args.steps, warmup=args.warmup)
        line = {"metric": METRIC, "value": cb["value"], "unit": "atom-evals/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "impl": "reference",
                "config": {"workload": WORKLOAD, "natoms": N, "nstruc": len(structs), "sample": cb["sample"]},
                "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": cb["value"], "unit": "atom-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    from ann_gb300 import FP64, MIXED, Context

    dev = local if world > 1 else 0
    torch.cuda.set_device(dev)
    ctx = Context(device=dev, precision=MIXED, use_graphs=True)
    ctx.load_text(WL.config_potential_text(2))
    WL.precondition(ctx, offs, posn, types, cell)
    import tempfile
    with tempfile.TemporaryDirectory() as td:
        p = Path(td) / "pot.ann"
        ctx.write(p)
        pot_text = p.read_text()
    ctx.load_text(pot_text)

    # ---- accuracy of the mixed path vs the FP64 path on the same batch
    E64, F64, W64 = ctx.compute(offs, posn, types, cell, precision=FP64)
    Emx, Fmx, Wmx = ctx.compute(offs, posn, types, cell, precision=MIXED)
    nat = np.diff(offs)
    acc_fp64 = {"e_mev_atom_max": float(np.max(np.abs(Emx - E64) / nat) * 1e3),
                "f_mev_A_max": float(np.max(np.abs(Fmx - F64)) * 1e3),
                "f_mev_A_rms": float(np.sqrt(np.mean((Fmx - F64) ** 2)) * 1e3),
                "reference": "plain FP64 GPU form on the same batch"}
    work = algorithmic_work(ctx, offs, posn, types, cell)

    # ---- launch shapes picked by the library's autotuner on this batch (outside the timed region,
    #      like the graph capture); the FP64 form gets its own when it is timed
    SHAPE_KEYS = ("tc_groups", "bp_blocks_per_sm", "nbr_blocks_per_sm")
    if args.no_tune:
        tuned = {"tc_groups": [0, 0, 0, 0], "bp_blocks_per_sm": 0, "nbr_blocks_per_sm": 0, "ms": None, "ms_default": None}
    else:
        ctx.compute(offs, posn, types, cell, precision=MIXED)
        tuned = ctx.autotune(precision=MIXED, reps=5)
    shapes = {k: tuned[k] for k in SHAPE_KEYS}

    timer = resident_timer(ctx, dev)

    def timed_device(prec, steps, warm):
        return timer(offs, posn, types, cell, prec, steps, warm)

    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    clocks = ClockSampler(dev)
    clocks.start()
    t_wall = time.perf_counter()
    ms = timed_device(MIXED, args.steps, W_)
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    ms_step = float(np.sum(ms) / len(ms))
    tmax = ms_step
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([ms_step], device=f"cuda:{dev}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        tmax = float(tt.item())
    value = N * world / (tmax * 1e-3)
    launches_per_step = ctx.kernels_per_batch()

    # ---- plain FP64 form on the same batch, with its own tuned shapes
    ctx.set_tuning()
    tuned64 = dict(tuned) if args.no_tune else ctx.autotune(precision=FP64, reps=1)
    ms64 = timed_device(FP64, max(3, args.steps // 4), 2)
    fp64_value = N / (float(np.mean(ms64)) * 1e-3)
    ctx.set_tuning(**shapes)

    # ---- per-phase kernel durations (CUDA events around each phase on the library stream)
    phase_ms = timer.phases(offs, posn, types, cell, MIXED, args.steps, W_)
    names = PHASES
    ph = np.array([phase_ms[n] for n in names])
    dom = int(np.argmax(ph))
    from ann_gb300.api import peaks
    pk = peaks()
    t_force = ph[4] * 1e-3
    sm_mhz = clk.get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count   # cudaDevAttrMultiProcessorCount
    fp32_peak = nsm * 128 * 2 * sm_mhz * 1e6 / 1e12           # TFLOP/s (FMA = 2 flop) at the sampled clock
    mufu_peak = nsm * 16 * sm_mhz * 1e6 / 1e12                 # T ops/s
    # DRAM bytes of one force-pass launch (ncu capture of this workload, committed under profiles/)
    traffic, traffic_src = None, None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        tr = json.loads(tf.read_text()).get("k_bp force pass (forces)")
        if tr:
            # the DRAM bytes of one force-pass launch as ncu measured them on this workload; another
            # batch scales them by its atoms (the traffic grows with the atom count at fixed density)
            traffic = float(tr["dram_bytes_per_launch"]) * N / float(tr["atoms_in_capture"])
            traffic_src = (f"{tr['dram_bytes_per_launch']} B per launch measured on {tr['atoms_in_capture']} atoms"
                           + ("" if N == tr["atoms_in_capture"] else f", scaled to {N} atoms") + f", from {tr['source']}")
    roofline = {"kernel": "k_bp force pass (" + names[4] + ")", "bound": "hbm",
                "achieved": work["force_bytes"] / t_force / 1e9, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": work["force_bytes"] / t_force / 1e9 / pk["hbm_gbs"], "traffic": traffic, "traffic_source": traffic_src,
                "algorithmic_bytes": work["force_bytes"], "peak_source": pk["source"], "dominant_phase": names[dom]}
    roofline_compute = {"kernel": roofline["kernel"], "bound": "fp32+mufu",
                        "fp32_tflops": work["force_flops"] / t_force / 1e12, "fp32_peak_tflops": fp32_peak,
                        "frac_fp32": work["force_flops"] / t_force / 1e12 / fp32_peak,
                        "mufu_tops": work["force_mufu"] / t_force / 1e12, "mufu_peak_tops": mufu_peak,
                        "frac_mufu": work["force_mufu"] / t_force / 1e12 / mufu_peak,
                        "note": f"peaks = {nsm} SMs (queried) x (128 FP32 lanes x 2 | 16 MUFU) x sampled SM clock; algorithmic counts "
                                "(angular pow = 2 MUFU) though the kernel replaces pow by squaring chains"}

    # ---- end to end through the C ABI: the batch in page-locked host memory (as a data loader
    #      delivers it), copied in and the energies / forces / virials copied out every step
    h_offs = ctx.pinned(offs.shape, np.int64); h_offs[:] = offs
    h_posn = ctx.pinned(posn.shape); h_posn[:] = posn
    h_types = ctx.pinned(types.shape, np.int32); h_types[:] = types
    h_cell = ctx.pinned(cell.shape); h_cell[:] = cell
    out = (ctx.pinned((len(structs),)), ctx.pinned((N, 3)), ctx.pinned((len(structs), 3, 3)))
    for _ in range(W_):
        ctx.compute(h_offs, h_posn, h_types, h_cell, precision=MIXED, out=out)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e, f, w = ctx.compute(h_offs, h_posn, h_types, h_cell, precision=MIXED, out=out)
    t_e2e = (time.perf_counter() - t0) / args.steps
    h2d = int(posn.nbytes + types.nbytes + cell.nbytes + 4 * len(offs) + 4 * N)
    d2h = int(8 * len(structs) + 24 * N + 72 * len(structs) + 32)

    line = {"metric": METRIC, "value": value, "unit": "atom-evals/s", "n_gpus": world, "steps": args.steps, "warmup": W_,
            "ms_per_step": tmax, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD, "natoms": N, "nstruc": len(structs), "precision": "mixed (FP32 basis/forces, BF16 hi/lo tensor-core networks with FP32 accumulation, FP64 energy sums)",
                       "l2": "flushed between steps (256 MiB write outside the timed events)", "graphs": True, "sm_count": nsm,
                       "launch_shapes": {"mixed": dict(shapes, ms=tuned["ms"], ms_default=tuned["ms_default"]),
                                         "fp64": {k: tuned64[k] for k in SHAPE_KEYS}},
                       "parallelism": f"replicas x{world} (structures sharded, no collective)"},
            "fp64_value": fp64_value, "speedup_vs_fp64": value / world / fp64_value,
            "accuracy_vs_fp64_gpu": acc_fp64, "phase_ms": phase_ms, "work": work,
            "roofline": roofline, "roofline_compute": roofline_compute,
            "e2e": {"value": N / t_e2e, "unit": "atom-evals/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": int(launches_per_step * args.steps),
            "clocks": clk, "wall_s_timed_region": t_wall}
    # the secondary GPU legs run before the oracle passes and the operand-form contexts: measured
    # after those, the fresh-batch training step read 0.65 ms against 0.53 ms alone (not explained)
    if rank == 0 and world == 1 and not args.no_extras:
        line["training"] = training_leg(dev)
        line["md"] = md_leg(dev)
        line["lammps"] = lammps_leg(dev)
    if rank == 0 and not args.no_parity:
        par, Eo, Fo = oracle_parity(offs, posn, types, cell, pot_text, E64, F64, W64, Emx, Fmx, Wmx)
        line["accuracy"] = dict(par["mixed_vs_oracle"], reference=par["reference"])
        line["parity"] = par
        if world == 1 and not args.no_extras:
            line["network_forms"] = network_forms_leg(dev, offs, posn, types, cell, pot_text, Eo, Fo)
    if rank == 0 and world == 1 and not args.no_extras:
        line["precision_study"] = precision_study_leg(dev)
        line["small_box"] = small_box_leg(dev)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_reference(offs, posn, types, cell, pot_text)
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
