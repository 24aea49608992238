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
ref_nnp.npz   : outputs of the reference's OWN potential code (src/nnp/nnp.cpp, nnh.cpp, type.cpp
                with the basis and network sources, compiled unmodified against oracle/ref_shim/
                into oracle/_ref/libref_nnp.so): three potentials read by NNP::read (a binary GAUSS
                potential with input scaling, the generic-basis potential of tests/cases.py, a
                ternary potential; all with vacuum energies) on periodic structures (random
                binary / ternary cells, cells smaller than rc, a triclinic cell, a lone atom,
                unwrapped coordinates), with the oracle's neighbour entries: NNP::symm's symmetry
                functions, NNP::energy, NNP::force with the Newton's-third-law reaction on every
                entry, the verlet::List NNP::force (reaction on untranslated entries only) and
                NNP::compute's energy; and the MD engine's ptnl::PotNNPE::compute
                (src/torch/pot_nnpe.cpp) on the same entries: its energy, and the largest
                difference of its forces from NNP::force's.
The reference keeps no golden vectors of its own (its tests print, seeded from the clock), so
these are the pins of the oracle's restatement.

Usage: python tests/golden/make_golden.py [--only basis|nn|nnp]
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
sys.path.insert(0, str(HERE.parents[1]))
from oracle_lib import Oracle, RefBasis, RefNN, RefNNP, eval_basisA, eval_basisR, nn_eval  # noqa: E402

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


def nnp_potentials():
    """(name, text) of the three potentials of ref_nnp.npz."""
    import cases
    from ann_gb300 import workloads as W

    def with_weights(text, names, nin, nodes, seed, scale_seed):
        params = [W.xavier_network(seed + 100 * t, nin, nodes) for t in range(len(names))]
        text = W.set_network_text(text, params, nin, nodes)
        rng = np.random.default_rng(scale_seed)
        out = []
        for line in text.splitlines():
            if line.startswith("inpw "):
                line = "inpw " + " ".join(f"{x:.15f}" for x in rng.uniform(0.05, 0.5, nin)) + " "
            elif line.startswith("inpb "):
                line = "inpb " + " ".join(f"{x:.15f}" for x in rng.uniform(-1.0, 0.0, nin)) + " "
            out.append(line)
        return "\n".join(out) + "\n"

    binary = with_weights(W.potential_text(["A", "B"], 6.5, 4, [0.003, 0.01], [12, 10, 1], "SOFTPLUS",
                                           energies={"A": -0.31, "B": 0.17}), ["A", "B"], 2 * 4 + 3 * 16, [12, 10, 1], 41, 42)
    ternary = with_weights(W.potential_text(["A", "B", "C"], 5.5, 3, [0.01], [8, 1], "TANH",
                                            energies={"A": -0.2, "B": 0.1, "C": 0.07}), ["A", "B", "C"], 3 * 3 + 6 * 8, [8, 1], 51, 52)
    return [("binary", binary), ("generic", cases.generic_potential_text(7)), ("ternary", ternary)]


def nnp_structures(name):
    """Periodic structures (posn, types, R with lattice vectors as columns) for one potential."""
    import cases
    from ann_gb300 import workloads as W
    rng = np.random.default_rng(SEED + 7)
    tiny = cases.tiny_cells()
    if name == "binary":
        return cases.small_binary(n_struc=2, seed=4) + tiny
    if name == "generic":
        return cases.small_binary(n_struc=1, seed=8) + tiny
    box = W.config4(seed=SEED + 9, dims=(5, 5, 4))
    R = np.array([[6.0, 1.2, 0.4], [0.0, 5.6, 0.9], [0.0, 0.0, 6.3]])
    x = rng.uniform(0, 1, (14, 3)) @ R.T
    return box + [(x, rng.integers(0, 3, 14).astype(np.int32), R)]


def main_nnp():
    import tempfile
    ref, orc = RefNNP(), Oracle()
    out = {}
    names = []
    k = 0
    for pi, (name, text) in enumerate(nnp_potentials()):
        names.append(name)
        out[f"pot_{name}"] = np.array(text)
        with tempfile.NamedTemporaryFile("w", suffix=".ann", delete=False) as f:
            f.write(text)
            path = f.name
        h = ref.read(path)
        rc = ref.L.ref_nnp_rc(h)
        hp = ref.potnnpe_read(path, rc)
        Path(path).unlink()
        assert ref.L.ref_nnp_nparams(h) == orc.load_text(text).nparams
        for x, t, R in nnp_structures(name):
            x = np.asarray(x, np.float64); t = np.asarray(t, np.int32); R = np.asarray(R, np.float64)
            i, j, img, _, _ = orc.neighbors(x, R, rc)
            G, E, F, Ec, Fc = ref.structure(h, t, x, R, i, j, img, newton=1, form=0)
            assert np.array_equal(F, Fc), "NNP::force and NNP::compute disagree"
            Gv, Ev, Fu, _, _ = ref.structure(h, t, x, R, i, j, img, newton=0, form=1)
            Gn, En, Fn, _, _ = ref.structure(h, t, x, R, i, j, img, newton=0, form=0)
            assert np.array_equal(Gv, G) and Ev == E and np.array_equal(Fn, Fu), "list forms disagree"
            Ep, Fp = ref.potnnpe_compute(hp, t, x, R, i, j, img)
            out.update({f"c{k}_pot": np.array(pi), f"c{k}_posn": x, f"c{k}_types": t, f"c{k}_R": R, f"c{k}_symm": G,
                        f"c{k}_energy": np.array(E), f"c{k}_force": F, f"c{k}_force_untranslated": Fu,
                        f"c{k}_energy_compute": np.array(Ec), f"c{k}_energy_potnnpe": np.array(Ep),
                        f"c{k}_force_potnnpe_vs_force": np.array(np.abs(Fp - F).max())})
            k += 1
        ref.L.ref_nnp_free(h)
        ref.L.ref_potnnpe_free(hp)
    out["pot_names"] = np.array(names)
    out["ncases"] = np.array(k)
    np.savez_compressed(HERE / "ref_nnp.npz", **out)
    print("wrote", HERE / "ref_nnp.npz", k, "structures")


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", choices=["basis", "nn", "nnp"])
    a = ap.parse_args()
    for part, fn in (("basis", main), ("nn", main_nn), ("nnp", main_nnp)):
        if a.only in (None, part):
            fn()
