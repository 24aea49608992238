"""Generate the golden fixtures of tests/golden/ (run here, where the reference sources are).

ref_basis.npz : outputs of the reference's OWN cutoff / radial / angular basis code and special
                functions (src/nnp/cutoff.cpp, basis_radial.cpp, basis_angular.cpp,
                src/math/special.cpp compiled unmodified by oracle/Makefile into
                oracle/_ref/libref_basis.so) at seeded sample points: Cutoff::cutf/cutg,
                BasisR::symm/force/symmd, BasisA::symm/force/symmd, fmexp, coscut, sincut.
ref_nn.npz    : outputs of the reference's OWN network code (src/ml/nn.cpp compiled unmodified
                against the plain-loop Eigen stand-in into oracle/_ref/libref_nn.so):
                ANN::resize's XAVIER initialisation (dist NORMAL) of three networks (the first
                64 parameters and a SHA-256 of all of them, little-endian doubles), and for
                networks of every activation with unit and with general input / output scaling,
                ANN::fpbp2's output, DODZ::grad's dO/dI, Cost::grad's dO/dp and D2ODZDI::grad's
                d2O/(dp dI), the latter projected on a fixed random input direction u (and in
                full for two cases).
The reference keeps no golden vectors of its own (its tests print, seeded from the clock), so
these are the pins of the oracle's restatement.

Usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
from oracle_lib import RefBasis, RefNN, eval_basisA, eval_basisR, nn_eval  # noqa: E402

SEED = 20261203


def main():
    ref = RefBasis()
    L = ref.L
    rng = np.random.default_rng(SEED)
    out = {}
    x = np.concatenate([rng.uniform(-745.0, 709.0, 400), rng.uniform(-5, 5, 200), [0.0, -1e-300, 1e-300]])
    out["fmexp_x"] = x
    out["fmexp_y"] = np.array([L.ref_fmexp(float(v)) for v in x])
    t = rng.uniform(0.0, np.pi, 200)
    out["cut_x"] = t
    out["coscut_y"] = np.array([L.ref_coscut(float(v)) for v in t])
    out["sincut_y"] = np.array([L.ref_sincut(float(v)) for v in t])
    # cutoffs
    rows = []
    for name in range(1, 5):
        for dr in rng.uniform(0.0, 7.0, 60):
            import ctypes as C
            f, g = C.c_double(), C.c_double()
            assert L.ref_cutoff(name, 6.0, float(dr), C.byref(f), C.byref(g)) == 0
            rows.append((name, 6.0, dr, f.value, g.value))
    out["cutoff"] = np.array(rows)
    # radial: per (function, cutoff) 30 points of 4 functions
    R_in, R_out = [], []
    for name in range(1, 7):
        for cut in range(1, 5):
            for _ in range(30):
                rs = rng.uniform(0.0, 3.0, 4); eta = rng.uniform(0.1, 2.0, 4)
                dr = float(rng.uniform(0.5, 7.0)); dE = rng.normal(size=4)
                s, amp, sd = eval_basisR(L, "ref_", cut, 6.0, name, rs, eta, dr, dE)
                R_in.append(np.concatenate([[name, cut, 6.0, dr], rs, eta, dE]))
                R_out.append(np.concatenate([s, [amp], sd]))
    out["radial_in"] = np.array(R_in)
    out["radial_out"] = np.array(R_out)
    # angular: eta in two groups (exercises the rflag grouping), integer and real zeta
    A_in, A_out = [], []
    for name in range(1, 7):
        for cut in range(1, 5):
            for _ in range(30):
                e = rng.uniform(1.0, 12.0, 2)
                eta = np.array([e[0], e[0], e[1], e[1]])
                zeta = rng.choice([1.0, 2.0, 4.0, 8.0, 1.5, 3.3], 4)
                lam = rng.choice([-1, 1], 4).astype(np.int32)
                dij, dik = rng.uniform(0.5, 7.0, 2); cs = float(rng.uniform(-1.0, 1.0)); dE = rng.normal(size=4)
                s, phi, e2, sd = eval_basisA(L, "ref_", cut, 6.0, name, eta, zeta, lam, float(dij), float(dik), cs, dE)
                A_in.append(np.concatenate([[name, cut, 6.0, dij, dik, cs], eta, zeta, lam, dE]))
                A_out.append(np.concatenate([s, [phi], e2, sd]))
    out["angular_in"] = np.array(A_in)
    out["angular_out"] = np.array(A_out)
    np.savez_compressed(HERE / "ref_basis.npz", **out)
    print("wrote", HERE / "ref_basis.npz", {k: v.shape for k, v in out.items()})
    main_nn()


# activation names in the order of NN::Neuron::Type (nn.hpp:84-103, values 1..19)
NEURONS = ["LINEAR", "SIGMOID", "TANH", "ISRU", "ARCTAN", "RELU", "ELU", "TANHRE", "SQRE", "SWISH", "GELU", "MISH",
           "PFLU", "SERF", "LOGISH", "SOFTPLUS", "SQPLUS", "ATISH", "TEST"]
NN_NIN, NN_NODES = 10, [8, 6, 1]


def main_nn():
    import ctypes as C
    ref = RefNN()
    L = ref.L
    rng = np.random.default_rng(SEED + 1)
    out = {}
    # initialisation: ANN::resize with XAVIER weights, NORMAL distribution, sigma_b 0.001, sigma_w 1
    for k, (nin, nodes, seed) in enumerate(((72, [64, 64, 1], 1234), (16, [20, 20, 1], 7), (96, [128, 128, 1], 99))):
        h = ref.create(nin, nodes, 16, init=4, seed=seed, dist=3)
        prm = ref.params(h)
        out[f"init{k}_shape"] = np.array([nin, seed] + nodes)
        out[f"init{k}_head"] = prm[:64]
        out[f"init{k}_sha256"] = np.frombuffer(hashlib.sha256(prm.astype("<f8").tobytes()).digest(), np.uint8)
        L.ref_nn_free(h)
    # evaluations: every activation, unit and general scaling
    rows = []          # neuron, c, scaled flag
    P = NN_NIN * NN_NODES[0] + NN_NODES[0] * NN_NODES[1] + NN_NODES[1] * NN_NODES[2] + sum(NN_NODES)
    params, scal, xs, us, outs, dodis, grads, d2us = [], [], [], [], [], [], [], []
    full = {}
    for ni, name in enumerate(NEURONS):
        for scaled in (0, 1):
            c = 1.3
            h = ref.create(NN_NIN, NN_NODES, ni + 1, c=c, init=4, seed=300 + 2 * ni + scaled, dist=3)
            p = ref.params(h)
            inpw = rng.uniform(0.3, 1.2, NN_NIN) if scaled else np.ones(NN_NIN)
            inpb = rng.uniform(-0.5, 0.5, NN_NIN) if scaled else np.zeros(NN_NIN)
            outw, outb = (0.7, -0.2) if scaled else (1.0, 0.0)
            _D = C.POINTER(C.c_double)
            L.ref_nn_set_scaling(h, inpw.ctypes.data_as(_D), inpb.ctypes.data_as(_D), outw, outb)
            x = rng.normal(0.0, 1.0, NN_NIN)
            u = rng.normal(0.0, 1.0, NN_NIN)
            o, dodi, gr, d2 = nn_eval(L, "ref_nn_eval", h, NN_NIN, P, x)
            rows.append((ni + 1, c, scaled))
            params.append(p); scal.append(np.concatenate([inpw, inpb, [outw, outb]])); xs.append(x); us.append(u)
            outs.append(o); dodis.append(dodi); grads.append(gr); d2us.append(d2 @ u)
            if (name, scaled) in (("TANH", 0), ("SOFTPLUS", 1)):
                full[f"d2full_{name}_{scaled}"] = d2
            L.ref_nn_free(h)
    out.update(nn_cases=np.array(rows), nn_params=np.array(params), nn_scaling=np.array(scal), nn_x=np.array(xs), nn_u=np.array(us),
               nn_out=np.array(outs), nn_dodi=np.array(dodis), nn_grad=np.array(grads), nn_d2u=np.array(d2us),
               nn_shape=np.array([NN_NIN] + NN_NODES), **full)
    np.savez_compressed(HERE / "ref_nn.npz", **out)
    print("wrote", HERE / "ref_nn.npz", {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
