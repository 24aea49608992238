"""Seeded structure / potential cases shared by the GPU parity tests."""
from __future__ import annotations

import numpy as np

from ann_gb300 import workloads as W
from ann_gb300.api import pack_batch

GENERIC_POTENTIAL = """ann
ntypes 2
name X mass 12.000000 energy -0.250000
name Y mass 16.000000 energy 0.125000
rc 5.000000
basis X
basis_radial X
BasisR TANH 5.000000 SECH 3
\t0.500000 1.200000
\t1.500000 0.800000
\t2.500000 1.500000
basis_radial Y
BasisR TANH 5.000000 LOGISTIC 2
\t1.000000 1.000000
\t2.000000 0.700000
basis_angular X X
BasisA TANH 5.000000 GAUSS2 3
\t3.000000 1.000000 1 0
\t3.000000 2.500000 -1 0
\t4.000000 3.000000 1 0
basis_angular X Y
BasisA TANH 5.000000 SECH 2
\t2.500000 1.500000 1 0
\t3.500000 2.000000 -1 0
basis_angular Y Y
BasisA TANH 5.000000 STUDENT3 2
\t2.000000 1.000000 1 0
\t2.000000 4.000000 -1 0
basis Y
basis_radial X
BasisR POLY3 5.000000 LOGCOSH 2
\t1.000000 1.100000
\t2.000000 0.900000
basis_radial Y
BasisR POLY3 5.000000 TANH 2
\t1.500000 1.300000
\t3.000000 0.600000
basis_angular X X
BasisA POLY3 5.000000 STUDENT4 2
\t2.500000 1.000000 1 0
\t3.000000 2.000000 -1 0
basis_angular X Y
BasisA POLY3 5.000000 STUDENT5 1
\t3.000000 1.700000 1 0
basis_angular Y Y
BasisA POLY3 5.000000 GAUSS 3
\t4.000000 1.300000 1 0
\t4.000000 2.000000 -1 0
\t5.000000 1.000000 1 0
nn X
nn 12 7 5 1
neuron SIGMOID 1.300000
inpw {inpw12}
outw 0.700000000000000
inpb {inpb12}
outb 0.300000000000000
bias[1] {b1}
bias[2] {b2}
bias[3] {b3}
weight[0,1] {w1}
weight[1,2] {w2}
weight[2,3] {w3}
nn Y
nn 10 6 1
neuron TANH 0.800000
inpw {inpw10}
outw 1.100000000000000
inpb {inpb10}
outb -0.200000000000000
bias[1] {c1}
bias[2] {c2}
weight[0,1] {v1}
weight[1,2] {v2}
"""


def _fmt(v):
    return " ".join(f"{x:.15f}" for x in v) + " "


def generic_potential_text(seed=7) -> str:
    """Every non-GAUSS angular variant, all radial variants but GAUSSIAN, TANH/POLY3 cutoffs,
    non-integer zeta, SIGMOID/TANH networks and vacuum energies (the reference's generic path)."""
    rng = np.random.default_rng(seed)
    return GENERIC_POTENTIAL.format(
        inpw12=_fmt(rng.uniform(0.5, 1.5, 12)), inpb12=_fmt(rng.uniform(-0.5, 0.5, 12)),
        b1=_fmt(rng.normal(0, 0.1, 7)), b2=_fmt(rng.normal(0, 0.1, 5)), b3=_fmt(rng.normal(0, 0.1, 1)),
        w1=_fmt(rng.normal(0, 0.5, 7 * 12)), w2=_fmt(rng.normal(0, 0.5, 5 * 7)), w3=_fmt(rng.normal(0, 0.5, 5)),
        inpw10=_fmt(rng.uniform(0.5, 1.5, 10)), inpb10=_fmt(rng.uniform(-0.5, 0.5, 10)),
        c1=_fmt(rng.normal(0, 0.1, 6)), c2=_fmt(rng.normal(0, 0.1, 1)),
        v1=_fmt(rng.normal(0, 0.5, 6 * 10)), v2=_fmt(rng.normal(0, 0.5, 6)))


NEURONS = ["LINEAR", "SIGMOID", "TANH", "ISRU", "ARCTAN", "RELU", "ELU", "TANHRE", "SQRE", "SWISH", "GELU", "MISH",
           "PFLU", "SERF", "LOGISH", "SOFTPLUS", "SQPLUS", "ATISH", "TEST"]     # nn.hpp:84-103, enum values 1..19


def activation_potential_text(neuron: str, c: float = 1.3, seed: int = 5) -> str:
    """A small binary potential (4 radial per species, 2x8 angular per pair: 32 inputs, 32-12-10-1
    networks) whose hidden layers use the given activation with scale c; Xavier weights, input
    scaling that keeps the pre-activations near the activation's curved part."""
    text = W.potential_text(["A", "B"], 6.5, 4, [0.003, 0.01], [12, 10, 1], neuron)
    nin = 2 * 4 + 3 * 2 * 8
    params = [W.xavier_network(seed + 100 * t, nin, [12, 10, 1]) for t in range(2)]
    text = W.set_network_text(text, params, nin, [12, 10, 1])
    text = text.replace(f"neuron {neuron} 1.000000", f"neuron {neuron} {c:f}")
    rng = np.random.default_rng(seed)
    out = []
    for line in text.splitlines():
        if line.startswith("inpw "):
            line = "inpw " + _fmt(rng.uniform(0.02, 0.2, nin))
        elif line.startswith("inpb "):
            line = "inpb " + _fmt(rng.uniform(-2.0, 0.0, nin))
        out.append(line)
    return "\n".join(out) + "\n"


def single_network_text(nin, nodes, neuron, c, inpw, inpb, outw, outb):
    """A one-type potential whose network has nin inputs (nin - 8 radial functions and 8 angular
    ones), the given hidden / output widths, activation (name) with scale c, and input / output
    scaling written with 17 significant digits (read back exactly)."""
    text = W.potential_text(["A"], 6.0, nin - 8, [0.01], list(nodes), neuron)
    text = text.replace(f"neuron {neuron} 1.000000", f"neuron {neuron} {c:.17g}")
    out = []
    for line in text.splitlines():
        if line.startswith("inpw "):
            line = "inpw " + " ".join(f"{v:.17g}" for v in inpw)
        elif line.startswith("inpb "):
            line = "inpb " + " ".join(f"{v:.17g}" for v in inpb)
        elif line.startswith("outw "):
            line = f"outw {outw:.17g}"
        elif line.startswith("outb "):
            line = f"outb {outb:.17g}"
        out.append(line)
    return "\n".join(out) + "\n"


def config_potential(ctx, cfg, tmp_path, precondition_batch=None):
    """Initialise the configuration potential in ctx, round-trip it through the 'ann' text format
    (what both sides read) and return that text."""
    W.make_potential(ctx, cfg)
    if precondition_batch is not None:
        W.precondition(ctx, *precondition_batch)
    p = tmp_path / f"pot{cfg}.ann"
    ctx.write(p)
    text = p.read_text()
    ctx.load_text(text)
    return text


def small_binary(n_struc=6, seed=11):
    s = W.random_binary(n_struc, 32, 160, seed=seed)
    return s


def ternary_box(dims=(10, 10, 6), seed=5):
    return W.config4(seed=seed, dims=dims)


def tiny_cells():
    """Cells smaller than the cutoff (many images), a triclinic cell, a lone atom (only self
    images) and unwrapped coordinates."""
    rng = np.random.default_rng(3)
    out = []
    out.append((np.array([[0.1, 0.2, 0.3], [1.6, 1.5, 1.4]]), np.array([0, 1], np.int32), np.eye(3) * 3.1))
    R = np.array([[4.0, 1.0, 0.5], [0.0, 3.8, 0.7], [0.0, 0.0, 4.2]])
    x = rng.uniform(0, 1, (5, 3)) @ R.T
    out.append((x, np.array([0, 1, 0, 1, 1], np.int32), R))
    out.append((np.array([[0.3, 0.2, 0.1]]), np.array([0], np.int32), np.eye(3) * 3.7))
    x = rng.uniform(0, 6, (6, 3))
    x[0] += np.array([6.0, 0, 0]) * 2
    x[1] -= np.array([0, 6.0, 0]) * 3
    out.append((x, np.array([0, 1, 1, 0, 0, 1], np.int32), np.eye(3) * 6.0))
    return out


def batch(structs):
    return pack_batch(structs)


# ---- the reference's argon example (examples/Ar): basis_Ar restated in the current file format
AR_RS = [0.00, 0.16, 0.31, 0.47, 0.63, 0.78, 0.94, 1.10, 1.25, 1.41]
AR_ETA = [0.016, 0.032, 0.054, 0.084, 0.126, 0.190, 0.287, 0.455, 0.760, 1.400]
AR_AETA = [0.120, 0.060, 0.030]


def argon_example_potential(rc=8.0, nodes=(7, 4, 2, 1), neuron="TANH", evac=-574.641, seed=3, sigma_w=0.5):
    """The example's argon potential: examples/Ar/basis_Ar (10 radial G2 (rs, eta), 3 angular G4
    (eta, zeta 5, lambda -1)) written in the current 'ann' format (BasisR GAUSSIAN takes
    exp(-(eta'(r-rs))^2), so eta' = sqrt(eta); BasisA GAUSS takes exp(-(rij^2+rik^2)/eta'^2), so
    eta' = 1/sqrt(eta)); nh 7 4 2 and the vacuum energy of nn_pot_train_init.txt; XAVIER normal
    weights. rc is 8 A rather than the example's 10 A: the FP64 rows of the densest training cell
    at 10 A exceed a block's shared memory."""
    nin = len(AR_RS) + len(AR_AETA)
    out = ["ann", "ntypes 1", f"name Ar mass 39.948000 energy {evac:f} ", f"rc {rc:f}", "basis Ar", "basis_radial Ar",
           f"BasisR COS {rc:f} GAUSSIAN {len(AR_RS)}"]
    out += [f"\t{r:f} {np.sqrt(e):f}" for r, e in zip(AR_RS, AR_ETA)]
    out += ["basis_angular Ar Ar", f"BasisA COS {rc:f} GAUSS {len(AR_AETA)}"]
    out += [f"\t{1 / np.sqrt(e):f} 5.000000 -1 0" for e in AR_AETA]
    out += ["nn Ar", "nn " + " ".join(map(str, [nin] + list(nodes))) + " ", f"neuron {neuron} 1.000000",
            "inpw " + " ".join(["1.000000000000000"] * nin) + " ", "outw 1.000000000000000 ",
            "inpb " + " ".join(["0.000000000000000"] * nin) + " ", "outb 0.000000000000000 "]
    prev = nin
    for l, n in enumerate(nodes):
        out.append(f"bias[{l + 1}] " + " ".join(["0.0"] * n) + " ")
    for l, n in enumerate(nodes):
        out.append(f"weight[{l},{l + 1}] " + " ".join(["0.0"] * (n * prev)) + " ")
        prev = n
    text = "\n".join(out) + "\n"
    return W.set_network_text(text, [W.xavier_network(seed, nin, list(nodes), 0.001, sigma_w)], nin, list(nodes))


def argon_example_data():
    """(train, val) batches of the fixture built from the example's QE outputs:
    each (offs, posn, types, cell, energies, forces)."""
    from pathlib import Path
    d = np.load(Path(__file__).resolve().parent / "golden" / "ar_qe.npz")
    out = []
    for k in ("train", "val"):
        X, C = d[k + "_posn"], d[k + "_cell"]
        b = pack_batch([(X[s], np.zeros(X.shape[1], np.int32), C[s]) for s in range(len(X))])
        out.append((*b, d[k + "_energy"], d[k + "_forces"].reshape(-1, 3)))
    return out
