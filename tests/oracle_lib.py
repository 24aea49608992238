"""ctypes access to the test-only CPU checkers under oracle/ (never used by the product).

- ``Oracle``: the FP64 restatement of the reference path (oracle/ann_oracle.cpp).
- ``RefBasis``: the reference's own cutoff / basis / special-function code compiled from its
  sources (oracle/_ref/libref_basis.so), present only where the reference sources are.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
ORACLE_DIR = ROOT / "oracle"
ORACLE_SO = ORACLE_DIR / "_build" / "libann_oracle.so"
REF_SO = ORACLE_DIR / "_ref" / "libref_basis.so"
REF_NN_SO = ORACLE_DIR / "_ref" / "libref_nn.so"
REF_NNP_SO = ORACLE_DIR / "_ref" / "libref_nnp.so"
ORACLE_TIMED_SO = ORACLE_DIR / "_build" / "libann_oracle_timed.so"


def _reference_src() -> Path:
    """The reference's src/ directory: ANN_REFERENCE_SRC, else the oracle recipe's default."""
    env = os.environ.get("ANN_REFERENCE_SRC")
    if env:
        return Path(env)
    try:
        out = subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), "print-ref"], capture_output=True, text=True, check=True)
        return Path(out.stdout.strip())
    except (OSError, subprocess.CalledProcessError):
        return Path(os.devnull) / "missing"


REF_SRC = _reference_src()

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_L = C.POINTER(C.c_longlong)


def _d(a):
    return None if a is None else a.ctypes.data_as(_D)


def _i(a):
    return None if a is None else a.ctypes.data_as(_I)


def _l(a):
    return None if a is None else a.ctypes.data_as(_L)


def build_oracle(ref: bool = False) -> None:
    target = ["oracle"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), *target], check=True)


class Oracle:
    """timed=True loads the build with the reference's optimisation flags and FP contraction
    (for timing the CPU baseline only; its results may differ in the last bits)."""

    def __init__(self, timed: bool = False):
        so = ORACLE_TIMED_SO if timed else ORACLE_SO
        if not so.exists() or so.stat().st_mtime < (ORACLE_DIR / "ann_oracle.cpp").stat().st_mtime:
            build_oracle()
        L = self.L = C.CDLL(str(so))
        L.orc_last_error.restype = C.c_char_p
        L.orc_load_text.restype = C.c_void_p
        L.orc_load_text.argtypes = [C.c_char_p]
        L.orc_free.argtypes = [C.c_void_p]
        for f in ("orc_ntypes", "orc_nparams"):
            getattr(L, f).argtypes = [C.c_void_p]
        L.orc_ninput.argtypes = [C.c_void_p, C.c_int]
        L.orc_rc.argtypes = [C.c_void_p]
        L.orc_rc.restype = C.c_double
        L.orc_get_params.argtypes = [C.c_void_p, _D]
        L.orc_set_params.argtypes = [C.c_void_p, _D]
        for f in ("orc_fmexp", "orc_coscut", "orc_sincut"):
            getattr(L, f).restype = C.c_double
            getattr(L, f).argtypes = [C.c_double]
        L.orc_cutoff.argtypes = [C.c_int, C.c_double, C.c_double, _D, _D]
        L.orc_activate.argtypes = [C.c_int, C.c_double, C.c_double, _D, _D, _D]
        L.orc_nn_eval.argtypes = [C.c_void_p, C.c_int, _D, _D, _D, _D, _D]
        L.orc_nn_size.argtypes = [C.c_void_p, C.c_int]
        L.orc_basisR.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, _D, _D, C.c_double, _D, _D, _D, _D]
        L.orc_basisA.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, _D, _D, _I, C.c_double, C.c_double, C.c_double, _D, _D, _D, _D, _D]
        L.orc_neighbors.restype = C.c_longlong
        L.orc_neighbors.argtypes = [C.c_int, _D, _D, C.c_double, C.c_longlong, _I, _I, _I, _D, _D, C.c_int]
        L.orc_compute.argtypes = [C.c_void_p, C.c_int, _L, _D, _I, _D, _D, _D, _D, _D, _D, C.c_int, C.c_int, C.c_int]
        L.orc_train.argtypes = [C.c_void_p, C.c_int, _L, _D, _I, _D, _D, _D, C.c_double, C.c_double, _D, _D]
        L.orc_error_cost_o1.argtypes = [C.c_void_p, C.c_int, _L, _D, _I, _D, _D, _D, _D]
        L.orc_error_cost_o1_ex.argtypes = [C.c_void_p, C.c_int, _L, _D, _I, _D, _D, C.c_int, C.c_int, C.c_double, _D, _D]
        L.orc_train_ex.argtypes = [C.c_void_p, C.c_int, _L, _D, _I, _D, _D, _D, C.c_double, C.c_double, C.c_int, C.c_int, C.c_double, _D, _D,
                                   C.c_int]
        L.orc_symm_jvp.argtypes = [C.c_void_p, C.c_int, _L, _D, _I, _D, _D, _D, C.c_int]
        L.orc_lj.restype = C.c_double
        L.orc_lj.argtypes = [C.c_int, _D, _D, C.c_double, C.c_double, C.c_double, _D]
        L.orc_md_step.argtypes = [C.c_void_p, C.c_int, _D, _D, _I, _D, _D, C.c_double, _D, _D, _D]
        L.orc_input_stats.restype = None
        L.orc_input_stats.argtypes = [C.c_int, _I, C.c_longlong, _I, _D, C.c_int, _D, C.POINTER(C.c_longlong)]
        L.orc_precondition.argtypes = [C.c_int, _D, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _D, _D]
        L.orc_taylor_perturb.restype = C.c_longlong
        L.orc_taylor_perturb.argtypes = [C.c_int, _L, _D, _D, _D, C.c_int, C.c_int, C.c_double, C.c_uint, _D, _L, _D, _D, _I]

    def err(self):
        return self.L.orc_last_error().decode()

    # ---- potential
    def load_text(self, text: str):
        p = self.L.orc_load_text(text.encode())
        if not p:
            raise RuntimeError(self.err())
        return Potential(self, p)

    # ---- geometry
    def activate(self, neuron: int, c: float, z: float):
        """(a, d, d2) of the oracle's activation (the reference's AFFPBP forms)."""
        a, d, d2 = np.zeros(1), np.zeros(1), np.zeros(1)
        if self.L.orc_activate(neuron, c, z, _d(a), _d(d), _d(d2)) != 0:
            raise ValueError(f"activation {neuron} not supported")
        return float(a[0]), float(d[0]), float(d2[0])

    def neighbors(self, x, R, rc, brute=False):
        """(i, j, image, r, d) of one structure; brute=True forces the all-pairs search."""
        x = np.ascontiguousarray(x, np.float64)
        Rc = np.ascontiguousarray(np.asarray(R, np.float64).T.reshape(9))
        n = len(x)
        cap = max(1024, n * 256)
        while True:
            i = np.zeros(cap, np.int32); j = np.zeros(cap, np.int32); img = np.zeros(3 * cap, np.int32)
            r = np.zeros(3 * cap); d = np.zeros(cap)
            k = self.L.orc_neighbors(n, _d(x), _d(Rc), rc, cap, _i(i), _i(j), _i(img), _d(r), _d(d), int(brute))
            if k >= 0:
                return i[:k], j[:k], img[:3 * k].reshape(-1, 3), r[:3 * k].reshape(-1, 3), d[:k]
            cap = -k

    def input_stats(self, nin, types, G):
        """Per-type input statistics (nnptefr2.cpp:686-775): (stats[T, 6, imax] with rows max, min,
        har, avg, dev, rms; counts[T])."""
        G = np.ascontiguousarray(G, np.float64)
        T, imax = len(nin), G.shape[1]
        out = np.zeros((T, 6, imax))
        cnt = np.zeros(T, np.int64)
        self.L.orc_input_stats(T, _i(np.ascontiguousarray(nin, np.int32)), len(types), _i(np.ascontiguousarray(types, np.int32)),
                               _d(G), imax, _d(out), cnt.ctypes.data_as(C.POINTER(C.c_longlong)))
        return out, cnt

    def precondition(self, stats_t, n, prebias, prescale, inbias=0.0, inscale=1.0):
        """(inpb, inpw) of one type from its statistics (nnptefr2.cpp:777-858)."""
        st = np.ascontiguousarray(stats_t, np.float64)
        b, w = np.zeros(n), np.zeros(n)
        if self.L.orc_precondition(n, _d(st), st.shape[1], prebias, prescale, inbias, inscale, _d(b), _d(w)) != 0:
            raise ValueError(self.err())
        return b, w

    def taylor_perturb(self, offs, posn, forces, energy, nadd, dist, rdelta, seed, rcov=None):
        """Perturbed training set (nnptefr2.cpp:2409-2479) with std::mt19937: (offs, posn, energy, src)."""
        offs = np.ascontiguousarray(offs, np.int64)
        x = np.ascontiguousarray(posn, np.float64)
        f = np.ascontiguousarray(forces, np.float64)
        e = np.ascontiguousarray(energy, np.float64)
        rc = None if rcov is None else np.ascontiguousarray(rcov, np.float64)
        args = (len(offs) - 1, _l(offs), _d(x), _d(f), _d(e), nadd, dist, rdelta, seed, _d(rc))
        ns = self.L.orc_taylor_perturb(*args, None, None, None, None)
        if ns < 0:
            raise ValueError("Invalid position distribution.")
        o = np.zeros(ns + 1, np.int64)
        self.L.orc_taylor_perturb(*args, _l(o), None, None, None)
        X = np.zeros((int(o[-1]), 3)); E = np.zeros(ns); S = np.zeros(ns, np.int32)
        self.L.orc_taylor_perturb(*args, _l(o), _d(X), _d(E), _i(S))
        return o, X, E, S

    def lj(self, x, R, eps=0.0104, sig=3.4, rcut=8.5):
        x = np.ascontiguousarray(x, np.float64)
        Rc = np.ascontiguousarray(np.asarray(R, np.float64).T.reshape(9))
        F = np.zeros_like(x)
        e = self.L.orc_lj(len(x), _d(x), _d(Rc), eps, sig, rcut, _d(F))
        return e, F


class Potential:
    def __init__(self, orc: Oracle, ptr):
        self.o, self.p = orc, C.c_void_p(ptr)
        self.L = orc.L

    def __del__(self):
        try:
            self.L.orc_free(self.p)
        except Exception:
            pass

    @property
    def ntypes(self):
        return self.L.orc_ntypes(self.p)

    @property
    def nparams(self):
        return self.L.orc_nparams(self.p)

    def ninput(self, t):
        return self.L.orc_ninput(self.p, t)

    def get_params(self):
        v = np.zeros(self.nparams)
        self.L.orc_get_params(self.p, _d(v))
        return v

    def set_params(self, v):
        v = np.ascontiguousarray(v, np.float64)
        self.L.orc_set_params(self.p, _d(v))

    def compute(self, offs, posn, types, cell, forces=True, symm=False, dedg=False, newton=1, nthreads=1):
        offs = np.ascontiguousarray(offs, np.int64)
        S = len(offs) - 1
        N = int(offs[-1])
        imax = max(self.ninput(t) for t in range(self.ntypes))
        E = np.zeros(S)
        F = np.zeros((N, 3)) if forces else None
        W = np.zeros((S, 3, 3)) if forces else None
        G = np.zeros((N, imax)) if symm else None
        D = np.zeros((N, imax)) if dedg else None
        rc = self.L.orc_compute(self.p, S, _l(offs), _d(np.ascontiguousarray(posn, np.float64)), _i(np.ascontiguousarray(types, np.int32)),
                                _d(np.ascontiguousarray(cell, np.float64)), _d(E), _d(F), _d(W), _d(G), _d(D), imax, newton, nthreads)
        if rc != 0:
            raise RuntimeError(self.o.err())
        return E, F, W, G, D

    def train(self, offs, posn, types, cell, e_ref, f_ref, wE=1.0, wF=0.1, loss=1, norm=1, delta=1.0, nthreads=1):
        """Loss (L, L_E, L_F) and dL/dp; loss 1 MSE, 2 MAE, 3 HUBER, 4 ASINH; norm 0 IDENTITY,
        1 LINEAR, 2 SQRT, 3 CBRT, 4 LOG (the energy term)."""
        offs = np.ascontiguousarray(offs, np.int64)
        lossv = np.zeros(3)
        g = np.zeros(self.nparams)
        rc = self.L.orc_train_ex(self.p, len(offs) - 1, _l(offs), _d(np.ascontiguousarray(posn, np.float64)),
                                 _i(np.ascontiguousarray(types, np.int32)), _d(np.ascontiguousarray(cell, np.float64)),
                                 _d(np.ascontiguousarray(e_ref, np.float64)), _d(np.ascontiguousarray(f_ref, np.float64)), wE, wF,
                                 loss, norm, delta, _d(lossv), _d(g), int(nthreads))
        loss = lossv
        if rc != 0:
            raise RuntimeError(self.o.err())
        return loss, g

    def error_cost_o1(self, offs, posn, types, cell, e_ref, loss=1, norm=1, delta=1.0):
        offs = np.ascontiguousarray(offs, np.int64)
        lossv = np.zeros(1)
        g = np.zeros(self.nparams)
        rc = self.L.orc_error_cost_o1_ex(self.p, len(offs) - 1, _l(offs), _d(np.ascontiguousarray(posn, np.float64)),
                                         _i(np.ascontiguousarray(types, np.int32)), _d(np.ascontiguousarray(cell, np.float64)),
                                         _d(np.ascontiguousarray(e_ref, np.float64)), loss, norm, delta, _d(lossv), _d(g))
        loss = lossv
        if rc != 0:
            raise RuntimeError(self.o.err())
        return loss[0], g

    def nn_eval(self, t, inp, d2=True):
        """(out, dO/dI, dO/dp, d2O/(dp dI)) of type t's network on one input (no vacuum energy)."""
        return nn_eval(self.L, "orc_nn_eval", self.p, self.ninput(t), self.L.orc_nn_size(self.p, t), inp, d2, t)

    def md_step(self, x, v, types, R, masses, dt, F):
        pe, ke = C.c_double(), C.c_double()
        Rc = np.ascontiguousarray(np.asarray(R, np.float64).T.reshape(9))
        rc = self.L.orc_md_step(self.p, len(types), _d(x), _d(v), _i(np.ascontiguousarray(types, np.int32)), _d(Rc),
                                _d(np.ascontiguousarray(masses, np.float64)), dt, _d(F), C.byref(pe), C.byref(ke))
        if rc != 0:
            raise RuntimeError(self.o.err())
        return pe.value, ke.value


def nn_eval(lib, fn, handle, nin, nparams, inp, d2=True, *pre):
    """(out, dO/dI, dO/dp, d2O/(dp dI) or None) of one network evaluation through the oracle
    (fn = "orc_nn_eval", pre = (type,)) or the reference build (fn = "ref_nn_eval")."""
    out = np.zeros(1); dodi = np.zeros(nin); g = np.zeros(nparams)
    d2o = np.zeros((nparams, nin)) if d2 else None
    rc = getattr(lib, fn)(handle, *pre, _d(np.ascontiguousarray(inp, np.float64)), _d(out), _d(dodi), _d(g), _d(d2o))
    if rc != 0:
        raise RuntimeError(f"{fn} failed")
    return out[0], dodi, g, d2o


class RefNN:
    """The reference's own network code (ml/nn.cpp compiled with the plain-loop Eigen stand-in)."""

    def __init__(self):
        if not REF_NN_SO.exists():
            if not REF_SRC.exists():
                raise FileNotFoundError("reference sources not available")
            build_oracle(ref=True)
        L = self.L = C.CDLL(str(REF_NN_SO))
        L.ref_nn_create.restype = C.c_void_p
        L.ref_nn_create.argtypes = [C.c_int, C.c_int, _I, C.c_int, C.c_double, C.c_int, C.c_int, C.c_double, C.c_double, C.c_int]
        L.ref_nn_free.argtypes = [C.c_void_p]
        L.ref_nn_size.argtypes = [C.c_void_p]
        L.ref_nn_get_params.argtypes = [C.c_void_p, _D]
        L.ref_nn_set_params.argtypes = [C.c_void_p, _D]
        L.ref_nn_set_scaling.argtypes = [C.c_void_p, _D, _D, C.c_double, C.c_double]
        L.ref_nn_eval.argtypes = [C.c_void_p, _D, _D, _D, _D, _D]
        L.ref_nn_last_error.restype = C.c_char_p

    def create(self, nin, nodes, neuron, c=1.0, init=4, seed=1, sigma_b=0.001, sigma_w=1.0, dist=1):
        nodes = np.ascontiguousarray(nodes, np.int32)
        h = self.L.ref_nn_create(nin, len(nodes), _i(nodes), neuron, c, init, seed, sigma_b, sigma_w, dist)
        if not h:
            raise RuntimeError(self.L.ref_nn_last_error().decode())
        return h

    def params(self, h):
        v = np.zeros(self.L.ref_nn_size(h))
        self.L.ref_nn_get_params(h, _d(v))
        return v


class RefNNP:
    """The reference's own potential code (nnp/nnp.cpp, nnh.cpp, type.cpp with the basis and
    network sources) compiled with the stand-ins of oracle/ref_shim/."""

    def __init__(self):
        if not REF_NNP_SO.exists():
            if not REF_SRC.exists():
                raise FileNotFoundError("reference sources not available")
            build_oracle(ref=True)
        L = self.L = C.CDLL(str(REF_NNP_SO))
        L.ref_nnp_last_error.restype = C.c_char_p
        L.ref_nnp_read.restype = C.c_void_p
        L.ref_nnp_read.argtypes = [C.c_char_p]
        for f in ("ref_nnp_free", "ref_nnp_ntypes", "ref_nnp_rc", "ref_nnp_nparams"):
            getattr(L, f).argtypes = [C.c_void_p]
        L.ref_nnp_rc.restype = C.c_double
        L.ref_nnp_ninput.argtypes = [C.c_void_p, C.c_int]
        L.ref_nnp_write.argtypes = [C.c_void_p, C.c_char_p]
        L.ref_nnp_domain.argtypes = [C.c_void_p, C.c_int, C.c_int, _I, _D, C.c_int, _I, _I, _D, _D]
        L.ref_potnnpe_read.restype = C.c_void_p
        L.ref_potnnpe_read.argtypes = [C.c_char_p, C.c_double]
        L.ref_potnnpe_free.argtypes = [C.c_void_p]
        L.ref_potnnpe_structure.argtypes = [C.c_void_p, C.c_int, _I, _D, _D, C.c_int, _I, _I, _I, C.c_int, _D, _D]
        L.ref_nnp_structure.argtypes = [C.c_void_p, C.c_int, _I, _D, _D, C.c_int, _I, _I, _I, C.c_int, C.c_int, C.c_int,
                                        _D, _D, _D, _D, _D]

    def read(self, path):
        h = self.L.ref_nnp_read(str(path).encode())
        if not h:
            raise RuntimeError(self.L.ref_nnp_last_error().decode())
        return C.c_void_p(h)

    def domain(self, h, nlocal, types, posn, ei, ej):
        """(E, F[nall]) of NNP on an MD engine's domain: nlocal centres then ghosts, the caller's
        neighbour entries (positions already shifted by their images)."""
        nall = len(types)
        E, F = np.zeros(1), np.zeros((nall, 3))
        rc = self.L.ref_nnp_domain(h, int(nlocal), nall, _i(np.ascontiguousarray(types, np.int32)),
                                   _d(np.ascontiguousarray(posn, np.float64)), len(ei), _i(np.ascontiguousarray(ei, np.int32)),
                                   _i(np.ascontiguousarray(ej, np.int32)), _d(E), _d(F))
        if rc != 0:
            raise RuntimeError(self.L.ref_nnp_last_error().decode())
        return float(E[0]), F

    def potnnpe_read(self, path, rc):
        """The MD engine's ptnl::PotNNPE reading a potential file (its cutoff set first, as the
        engine's pot line does)."""
        h = self.L.ref_potnnpe_read(str(path).encode(), float(rc))
        if not h:
            raise RuntimeError(self.L.ref_nnp_last_error().decode())
        return C.c_void_p(h)

    def potnnpe_compute(self, h, types, posn, R, ei, ej, img, newton=1):
        """(E, F) of PotNNPE::compute on one structure."""
        n = len(types)
        E, F = np.zeros(1), np.zeros((n, 3))
        Rc = np.ascontiguousarray(np.asarray(R, np.float64).T.reshape(9))
        rc = self.L.ref_potnnpe_structure(h, n, _i(np.ascontiguousarray(types, np.int32)), _d(np.ascontiguousarray(posn, np.float64)),
                                          _d(Rc), len(ei), _i(np.ascontiguousarray(ei, np.int32)), _i(np.ascontiguousarray(ej, np.int32)),
                                          _i(np.ascontiguousarray(img, np.int32)), int(newton), _d(E), _d(F))
        if rc != 0:
            raise RuntimeError(self.L.ref_nnp_last_error().decode())
        return float(E[0]), F

    def write(self, h, path):
        if self.L.ref_nnp_write(h, str(path).encode()) != 0:
            raise RuntimeError(self.L.ref_nnp_last_error().decode())

    def structure(self, h, types, posn, R, ei, ej, img, newton=1, form=0):
        """(symm, E, F, E_compute, F_compute) of one structure (R: lattice vectors as columns)."""
        n = len(types)
        width = max(self.L.ref_nnp_ninput(h, t) for t in range(self.L.ref_nnp_ntypes(h)))
        G = np.zeros((n, width)); F = np.zeros((n, 3)); Fc = np.zeros((n, 3))
        E, Ec = np.zeros(1), np.zeros(1)
        Rc = np.ascontiguousarray(np.asarray(R, np.float64).T.reshape(9))
        rc = self.L.ref_nnp_structure(h, n, _i(np.ascontiguousarray(types, np.int32)), _d(np.ascontiguousarray(posn, np.float64)),
                                      _d(Rc), len(ei), _i(np.ascontiguousarray(ei, np.int32)), _i(np.ascontiguousarray(ej, np.int32)),
                                      _i(np.ascontiguousarray(img, np.int32)), int(newton), int(form), width, _d(G), _d(E), _d(F),
                                      _d(Ec), _d(Fc))
        if rc != 0:
            raise RuntimeError(self.L.ref_nnp_last_error().decode())
        return G, float(E[0]), F, float(Ec[0]), Fc


class RefBasis:
    """The reference's own basis/cutoff/special functions (compiled from its sources)."""

    def __init__(self):
        if not REF_SO.exists():
            if not REF_SRC.exists():
                raise FileNotFoundError("reference sources not available")
            build_oracle(ref=True)
        L = self.L = C.CDLL(str(REF_SO))
        for f in ("ref_fmexp", "ref_coscut", "ref_sincut"):
            getattr(L, f).restype = C.c_double
            getattr(L, f).argtypes = [C.c_double]
        L.ref_cutoff.argtypes = [C.c_int, C.c_double, C.c_double, _D, _D]
        L.ref_basisR.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, _D, _D, C.c_double, _D, _D, _D, _D]
        L.ref_basisA.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, _D, _D, _I, C.c_double, C.c_double, C.c_double, _D, _D, _D, _D, _D]
        L.ref_read_basisR.argtypes = [C.c_char_p, _I, _D, _I, _I, _D, _D, C.c_int]
        L.ref_read_basisA.argtypes = [C.c_char_p, _I, _D, _I, _I, _D, _D, _I, _I, C.c_int]


def eval_basisR(lib, prefix, cut, rc, name, rs, eta, dr, dEdG):
    n = len(eta)
    s = np.zeros(n); sd = np.zeros(n); amp = C.c_double()
    f = getattr(lib, prefix + "basisR")
    assert f(cut, rc, name, n, _d(np.ascontiguousarray(rs, np.float64)), _d(np.ascontiguousarray(eta, np.float64)), dr, _d(s),
             _d(np.ascontiguousarray(dEdG, np.float64)), C.byref(amp), _d(sd)) == 0
    return s, amp.value, sd


def eval_basisA(lib, prefix, cut, rc, name, eta, zeta, lam, dij, dik, cs, dEdG):
    n = len(eta)
    s = np.zeros(n); sd = np.zeros(3 * n); phi = C.c_double(); e2 = np.zeros(2)
    f = getattr(lib, prefix + "basisA")
    assert f(cut, rc, name, n, _d(np.ascontiguousarray(eta, np.float64)), _d(np.ascontiguousarray(zeta, np.float64)),
             _i(np.ascontiguousarray(lam, np.int32)), dij, dik, cs, _d(s), _d(np.ascontiguousarray(dEdG, np.float64)), C.byref(phi),
             _d(e2), _d(sd)) == 0
    return s, phi.value, e2, sd
