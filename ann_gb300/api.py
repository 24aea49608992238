"""ctypes binding of the C ABI (include/ann_gpu.h) with numpy in and out.

``Context`` mirrors the reference's NNP usage (src/nnp/nnpce.cpp:273-287): load a potential
(NNP::read), then compute energies / forces of structures (NeighborList + NNP::symm +
NNP::compute / PotNNPE::compute). Errors raise AnnError with the library's message, the way the
reference raises std::invalid_argument / std::runtime_error.
"""
from __future__ import annotations

import ctypes as C
import weakref
import os
from pathlib import Path

import numpy as np

FP64 = 0
MIXED = 1
NEWTON_ALL_IMAGES = 0
NEWTON_UNTRANSLATED = 1

_HERE = Path(__file__).resolve().parent
_LIB = None


class AnnError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[ann error {code}] {msg}")
        self.code = code


class Options(C.Structure):
    _fields_ = [("device", C.c_int32), ("precision", C.c_int32), ("newton", C.c_int32), ("max_neighbors", C.c_int32),
                ("use_graphs", C.c_int32), ("mlp_backend", C.c_int32), ("tc_groups", C.c_int32), ("tc_split", C.c_int32)]


def library_path() -> Path:
    return Path(os.environ.get("ANN_GPU_LIB", _HERE / "libann_gpu.so"))


def build_library(verbose_ptxas: bool = False) -> Path:
    from .build import build
    return build(verbose_ptxas=verbose_ptxas)


_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_I64 = C.POINTER(C.c_int64)
_V = C.c_void_p

_SIGS = {
    "ann_default_options": (None, [C.POINTER(Options)]),
    "ann_create": (C.c_int, [C.POINTER(_V), C.POINTER(Options)]),
    "ann_destroy": (C.c_int, [_V]),
    "ann_last_error": (C.c_char_p, [_V]),
    "ann_abi_version": (C.c_int, []),
    "ann_load_potential": (C.c_int, [_V, C.c_char_p]),
    "ann_load_potential_text": (C.c_int, [_V, C.c_char_p]),
    "ann_write_potential": (C.c_int, [_V, C.c_char_p]),
    "ann_num_types": (C.c_int, [_V, _I32]),
    "ann_type_index": (C.c_int, [_V, C.c_char_p, _I32]),
    "ann_type_name": (C.c_int, [_V, C.c_int32, C.c_char_p, C.c_int32]),
    "ann_cutoff": (C.c_int, [_V, _D]),
    "ann_num_inputs": (C.c_int, [_V, C.c_int32, _I32]),
    "ann_num_params": (C.c_int, [_V, _I64]),
    "ann_network_form": (C.c_int, [_V, C.c_int32, _I32, _I32]),
    "ann_set_wait_limit": (C.c_int, [_V, C.c_int32]),
    "ann_get_params": (C.c_int, [_V, _D, C.c_int64]),
    "ann_set_params": (C.c_int, [_V, _D, C.c_int64]),
    "ann_set_input_scaling": (C.c_int, [_V, C.c_int32, _D, _D, C.c_int32]),
    "ann_init_network": (C.c_int, [_V, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double]),
    "ann_compute": (C.c_int, [_V, C.c_int32, _V, _V, _V, _V, _V, _V, _V, C.c_int32]),   # addresses (the per-call path)
    "ann_opt_set_schedule": (C.c_int, [_V, C.c_int32, C.c_double, C.c_int32, C.c_int32, C.c_double]),
    "ann_opt_init": (C.c_int, [_V, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_double]),
    "ann_opt_step": (C.c_int, [_V, C.c_double]),
    "ann_train_set_loss": (C.c_int, [_V, C.c_int32, C.c_int32, C.c_double]),
    "ann_host_alloc": (C.c_int, [_V, C.c_int64, C.POINTER(C.c_void_p)]),
    "ann_host_free": (C.c_int, [_V, C.c_void_p]),
    "ann_compute_list": (C.c_int, [_V, C.c_int32, _I32, _I32, _I32, C.c_int32, _D, _I32, _D, _D, _D, _D, C.c_int32, C.c_int32]),
    "ann_stats_reset": (C.c_int, [_V]),
    "ann_stats_accumulate": (C.c_int, [_V]),
    "ann_stats_get": (C.c_int, [_V, C.c_int32, _I64, _D]),
    "ann_precondition": (C.c_int, [_V, C.c_int32, C.c_int32, C.c_double, C.c_double]),
    "ann_get_input_scaling": (C.c_int, [_V, C.c_int32, _D, _D, C.c_int32]),
    "ann_batch_upload": (C.c_int, [_V, C.c_int32, _I64, _D, _I32, _D]),
    "ann_batch_set_device": (C.c_int, [_V, C.c_int32, _I64, _V, _V, _V]),
    "ann_batch_compute": (C.c_int, [_V, C.c_int32, C.c_int32]),
    "ann_batch_download": (C.c_int, [_V, _D, _D, _D]),
    "ann_batch_results_device": (C.c_int, [_V, _V, _V, _V]),
    "ann_synchronize": (C.c_int, [_V]),
    "ann_kernel_count": (C.c_int, [_V, _I64]),
    "ann_profile_phases": (C.c_int, [_V, C.c_int32]),
    "ann_phase_times": (C.c_int, [_V, _D, C.c_int32]),
    "ann_stream": (_V, [_V]),
    "ann_symm_width": (C.c_int, [_V, _I32]),
    "ann_get_symm": (C.c_int, [_V, _D, C.c_int64]),
    "ann_get_dedg": (C.c_int, [_V, _D, C.c_int64]),
    "ann_get_atom_energies": (C.c_int, [_V, _D, C.c_int64]),
    "ann_num_neighbors": (C.c_int, [_V, _I64]),
    "ann_get_neighbors": (C.c_int, [_V, _I32, _I32, _I32, _D, C.c_int64]),
    "ann_train_forward": (C.c_int, [_V, C.c_int32, _I64, _D, _I32, _D, _D, _D, C.c_double, C.c_double, C.c_int32, _D]),
    "ann_train_forward_staged": (C.c_int, [_V, C.c_double, C.c_double, C.c_int32, _D]),
    "ann_train_backward": (C.c_int, [_V, C.c_double, _D, C.c_int64]),
    "ann_adam_init": (C.c_int, [_V, C.c_double, C.c_double, C.c_double, C.c_double]),
    "ann_adam_step": (C.c_int, [_V, C.c_double]),
    "ann_md_init": (C.c_int, [_V, C.c_int64, _D, _D, _I32, _D, _D, C.c_double, C.c_double, C.c_int32]),
    "ann_md_run": (C.c_int, [_V, C.c_int32, _D, _D, _I32]),
    "ann_md_get_state": (C.c_int, [_V, _D, _D, _D]),
    "ann_network_noalloc": (C.c_int, [_V, C.c_int32, _V, _V, _V, _V, C.c_int32]),
    "ann_autotune": (C.c_int, [_V, C.c_int32, C.c_int32, _V]),
    "ann_set_tuning": (C.c_int, [_V, _V]),
}

ABI_SYMBOLS = tuple(_SIGS)


def peaks() -> dict:
    """Roofline denominators: the measured copy bandwidth / bf16 GEMM rate of the GB300s
    (MEASURED_PEAKS.json at the repository root), else the stated fallback."""
    import json
    p = _HERE.parent / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "bf16_tflops": float(d["bf16_tflops"]),
                "bf16_tflops_sustained": float(d.get("bf16_tflops_sustained", d["bf16_tflops"])),
                "sm_max_mhz": float(d.get("sm_max_mhz", 2070.0)), "source": "measured (MEASURED_PEAKS.json)"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0,
            "source": "fallback (6.8 TB/s, 1.9 PFLOP/s)"}


def load_library(path: str | Path | None = None):
    """Load libann_gpu.so (raises AnnError if it is missing: there is no fallback)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else library_path()
    if not p.exists():
        raise AnnError(-1, f"{p} not built: run `python -m ann_gb300.build` (the GPU path has no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def _d(a):
    return None if a is None else a.ctypes.data_as(_D)


def _i32(a):
    return None if a is None else a.ctypes.data_as(_I32)


def _i64(a):
    return None if a is None else a.ctypes.data_as(_I64)


def pack_batch(structures):
    """Pack a list of (posn[N,3], type[N], cell[3,3] with lattice vectors as columns) into the
    flat arrays of the C ABI: offsets[S+1] int64, posn[3N] f64, type[N] i32, cell[9S] f64
    (column-major: cell[9s + 3c + r] = R[r, c])."""
    offs = np.zeros(len(structures) + 1, dtype=np.int64)
    for s, (x, t, R) in enumerate(structures):
        offs[s + 1] = offs[s] + len(t)
    posn = np.ascontiguousarray(np.concatenate([np.asarray(x, dtype=np.float64).reshape(-1, 3) for x, _, _ in structures])
                                if structures else np.zeros((0, 3)), dtype=np.float64)
    types = np.ascontiguousarray(np.concatenate([np.asarray(t, dtype=np.int32) for _, t, _ in structures])
                                 if structures else np.zeros(0, dtype=np.int32), dtype=np.int32)
    cell = np.ascontiguousarray(np.stack([np.asarray(R, dtype=np.float64).T.reshape(9) for _, _, R in structures])
                                if structures else np.zeros((0, 9)), dtype=np.float64)
    return offs, posn, types, cell


class Tuning(C.Structure):
    """ann_tuning: launch shapes of the E+F sequence (0 = the built-in rule)."""
    _fields_ = [("tc_groups", C.c_int32 * 4), ("bp_blocks_per_sm", C.c_int32), ("nbr_blocks_per_sm", C.c_int32),
                ("ms", C.c_double), ("ms_default", C.c_double)]

    def as_dict(self) -> dict:
        return {"tc_groups": list(self.tc_groups), "bp_blocks_per_sm": self.bp_blocks_per_sm,
                "nbr_blocks_per_sm": self.nbr_blocks_per_sm, "ms": self.ms, "ms_default": self.ms_default}


class Context:
    """One device context: a loaded potential plus device buffers (one per host thread)."""

    def __init__(self, device: int = 0, precision: int = MIXED, newton: int = NEWTON_ALL_IMAGES, max_neighbors: int = 0,
                 use_graphs: bool = True, mlp_backend: int = 0, tc_groups: int = 0, tc_split: int = 0):
        self.lib = load_library()
        o = Options()
        self.lib.ann_default_options(C.byref(o))
        o.device, o.precision, o.newton, o.max_neighbors = device, precision, newton, max_neighbors
        o.use_graphs, o.mlp_backend, o.tc_groups, o.tc_split = int(use_graphs), mlp_backend, tc_groups, tc_split
        h = _V()
        rc = self.lib.ann_create(C.byref(h), C.byref(o))
        if rc != 0:
            raise AnnError(rc, self.lib.ann_last_error(None).decode())
        self.h = h
        self.precision = precision

    def close(self):
        if getattr(self, "h", None):
            self.lib.ann_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _ck(self, rc):
        if rc != 0:
            raise AnnError(rc, self.lib.ann_last_error(self.h).decode())

    # ---- potential
    def load(self, path):
        self._ck(self.lib.ann_load_potential(self.h, str(path).encode()))
        return self

    def load_text(self, text: str):
        self._ck(self.lib.ann_load_potential_text(self.h, text.encode()))
        return self

    def write(self, path):
        self._ck(self.lib.ann_write_potential(self.h, str(path).encode()))

    @property
    def ntypes(self) -> int:
        n = C.c_int32()
        self._ck(self.lib.ann_num_types(self.h, C.byref(n)))
        return n.value

    def type_index(self, name: str) -> int:
        n = C.c_int32()
        self._ck(self.lib.ann_type_index(self.h, name.encode(), C.byref(n)))
        return n.value

    def type_name(self, i: int) -> str:
        buf = C.create_string_buffer(256)
        self._ck(self.lib.ann_type_name(self.h, i, buf, 256))
        return buf.value.decode()

    @property
    def rc(self) -> float:
        v = C.c_double()
        self._ck(self.lib.ann_cutoff(self.h, C.byref(v)))
        return v.value

    def set_wait_limit(self, polls: int = -1):
        """ann_set_wait_limit: polls >= 0 makes the device waits give up after that many non-blocking
        polls (0: at once; testing the timeout path); -1 restores the built-in bounds."""
        self._ck(self.lib.ann_set_wait_limit(self.h, int(polls)))

    def network_form(self, t: int):
        """(backend, split) of the MIXED network pass for type t: backend 2 = tensor cores with
        split 1, 2 or 3, backend 1 = SIMT (split 0)."""
        b, s = C.c_int32(), C.c_int32()
        self._ck(self.lib.ann_network_form(self.h, t, C.byref(b), C.byref(s)))
        return b.value, s.value

    def num_inputs(self, t: int) -> int:
        n = C.c_int32()
        self._ck(self.lib.ann_num_inputs(self.h, t, C.byref(n)))
        return n.value

    @property
    def nparams(self) -> int:
        n = C.c_int64()
        self._ck(self.lib.ann_num_params(self.h, C.byref(n)))
        return n.value

    def get_params(self) -> np.ndarray:
        p = np.zeros(self.nparams)
        self._ck(self.lib.ann_get_params(self.h, _d(p), len(p)))
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float64)
        self._ck(self.lib.ann_set_params(self.h, _d(p), len(p)))

    def set_input_scaling(self, t: int, inpw, inpb):
        w = np.ascontiguousarray(inpw, dtype=np.float64)
        b = np.ascontiguousarray(inpb, dtype=np.float64)
        self._ck(self.lib.ann_set_input_scaling(self.h, t, _d(w), _d(b), len(w)))

    def init_network(self, t: int, seed: int, dist: int = 0, init: int = 4, sigma_b: float = 0.001, sigma_w: float = 1.0):
        self._ck(self.lib.ann_init_network(self.h, t, seed, dist, init, sigma_b, sigma_w))

    # ---- compute
    def pinned(self, shape, dtype=np.float64) -> np.ndarray:
        """A numpy array in page-locked host memory (ann_host_alloc), freed with the array: inputs
        and outputs there are copied by DMA without staging."""
        dt = np.dtype(dtype)
        nbytes = int(np.prod(shape)) * dt.itemsize
        ptr = C.c_void_p()
        self._ck(self.lib.ann_host_alloc(self.h, nbytes, C.byref(ptr)))
        if not ptr.value:
            return np.zeros(shape, dt)
        buf = (C.c_char * nbytes).from_address(ptr.value)
        arr = np.frombuffer(buf, dtype=dt).reshape(shape)
        weakref.finalize(buf, self.lib.ann_host_free, None, C.c_void_p(ptr.value))
        return arr

    def compute(self, offs, posn, types, cell, forces=True, virial=True, precision=None, out=None):
        """E (+F, virial) of a packed batch; returns (energy[S], forces[N,3] or None, virial[S,3,3] or None).
        out = (energy, forces, virial) arrays to write into (e.g. pinned ones), else new arrays."""
        prec = self.precision if precision is None else precision
        S = len(offs) - 1
        N = int(offs[-1])
        self._S, self._N = S, N
        if out is not None:
            e, f, w = out
            f = f if forces else None
            w = w if virial else None
        else:
            e = np.zeros(S)
            f = np.zeros((N, 3)) if forces else None
            w = np.zeros((S, 3, 3)) if virial else None
        o, x, t, c = (np.ascontiguousarray(offs, np.int64), np.ascontiguousarray(posn, np.float64),
                      np.ascontiguousarray(types, np.int32), np.ascontiguousarray(cell, np.float64))
        for arr in (e, f, w):
            if arr is not None and not (arr.dtype == np.float64 and arr.flags.c_contiguous):
                raise ValueError("out arrays must be C-contiguous float64")
        self._ck(self.lib.ann_compute(self.h, S, o.ctypes.data, x.ctypes.data, t.ctypes.data, c.ctypes.data, e.ctypes.data,
                                      None if f is None else f.ctypes.data, None if w is None else w.ctypes.data, prec))
        return e, f, w

    def compute_list(self, x, types, numneigh, neigh, ilist=None, forces=True, virial=True, eatom=False, precision=None,
                     keep=False, inum=None):
        """E (+F of all nall atoms, virial, per-row energies) from a full neighbour list over local and
        ghost atoms (the LAMMPS pair style shape, ann_compute_list). keep=True reuses the list, ilist
        and types of the previous call (ANN_LIST_KEEP; types / numneigh / neigh may be None and inum
        must then be given). Returns (energy, forces[nall,3] or None, virial[3,3] or None,
        eatom[inum] or None)."""
        prec = self.precision if precision is None else precision
        x = np.ascontiguousarray(x, np.float64).reshape(-1, 3)
        t = None if types is None else np.ascontiguousarray(types, np.int32)
        nn = None if numneigh is None else np.ascontiguousarray(numneigh, np.int32)
        nb = None if neigh is None else np.ascontiguousarray(neigh, np.int32)
        il = None if ilist is None else np.ascontiguousarray(ilist, np.int32)
        nall = len(x)
        inum = len(nn) if inum is None else int(inum)
        e = np.zeros(1)
        f = np.zeros((nall, 3)) if forces else None
        w = np.zeros((3, 3)) if virial else None
        ea = np.zeros(inum) if eatom else None
        self._ck(self.lib.ann_compute_list(self.h, inum, _i32(il), _i32(nn), _i32(nb), nall, _d(x), _i32(t), _d(e), _d(ea), _d(f),
                                           _d(w), prec, 1 if keep else 0))
        return e[0], f, w, ea

    # ---- input statistics and pre-conditioning (nnptefr2.cpp:686-858)
    PREBIAS = {"IDENTITY": 0, "MEAN": 1, "HAR": 2, "RMS": 3, "MID": 4, "MIN": 5}
    PRESCALE = {"IDENTITY": 0, "DEV": 1, "MINMAX": 2, "MAX": 3}

    def stats_reset(self):
        self._ck(self.lib.ann_stats_reset(self.h))

    def stats_accumulate(self):
        """Add the symmetry functions of the last computed batch to the statistics."""
        self._ck(self.lib.ann_stats_accumulate(self.h))

    def stats(self, t: int):
        """(count, stats[6, nInput]) of type t: rows max, min, har, avg, dev, rms."""
        n = self.num_inputs(t)
        out = np.zeros(6 * n)
        cnt = C.c_int64()
        self._ck(self.lib.ann_stats_get(self.h, t, C.byref(cnt), _d(out)))
        return cnt.value, out.reshape(6, n)

    def precondition(self, prebias="MEAN", prescale="DEV", inbias=0.0, inscale=1.0):
        pb = self.PREBIAS[prebias] if isinstance(prebias, str) else int(prebias)
        ps = self.PRESCALE[prescale] if isinstance(prescale, str) else int(prescale)
        self._ck(self.lib.ann_precondition(self.h, pb, ps, inbias, inscale))

    def input_scaling(self, t: int):
        """(inpw, inpb) of type t's network."""
        n = self.num_inputs(t)
        w, b = np.zeros(n), np.zeros(n)
        self._ck(self.lib.ann_get_input_scaling(self.h, t, _d(w), _d(b), n))
        return w, b

    def upload(self, offs, posn, types, cell):
        self._keep = [np.ascontiguousarray(offs, np.int64), np.ascontiguousarray(posn, np.float64),
                      np.ascontiguousarray(types, np.int32), np.ascontiguousarray(cell, np.float64)]
        o, x, t, c = self._keep
        self._S, self._N = len(o) - 1, int(o[-1])
        self._ck(self.lib.ann_batch_upload(self.h, self._S, _i64(o), _d(x), _i32(t), _d(c)))

    def compute_resident(self, precision=None, forces=True):
        self._ck(self.lib.ann_batch_compute(self.h, self.precision if precision is None else precision, int(forces)))

    def download(self, forces=True, virial=True):
        e = np.zeros(self._S)
        f = np.zeros((self._N, 3)) if forces else None
        w = np.zeros((self._S, 3, 3)) if virial else None
        self._ck(self.lib.ann_batch_download(self.h, _d(e), _d(f), _d(w)))
        return e, f, w

    def synchronize(self):
        self._ck(self.lib.ann_synchronize(self.h))

    @property
    def stream(self) -> int:
        return self.lib.ann_stream(self.h) or 0

    # ---- instrumentation
    def kernel_count(self) -> int:
        n = C.c_int64()
        self._ck(self.lib.ann_kernel_count(self.h, C.byref(n)))
        return n.value

    def kernels_per_batch(self, precision=None) -> int:
        """Kernels one resident-batch evaluation launches (graph replays count their nodes)."""
        k0 = self.kernel_count()
        self.compute_resident(precision)
        self.synchronize()
        return self.kernel_count() - k0

    def profile_phases(self, enable: bool):
        self._ck(self.lib.ann_profile_phases(self.h, int(enable)))

    def phase_times(self) -> np.ndarray:
        ms = np.zeros(6)
        self._ck(self.lib.ann_phase_times(self.h, _d(ms), 6))
        return ms

    # ---- launch shapes
    def autotune(self, precision=None, reps: int = 5) -> dict:
        """Time the run-time launch shapes on the staged batch (the last compute call's structures)
        and keep the fastest for later calls (ann_autotune); returns the choice and its time."""
        prec = self.precision if precision is None else precision
        t = Tuning()
        self._ck(self.lib.ann_autotune(self.h, prec, reps, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, tc_groups=(0, 0, 0, 0), bp_blocks_per_sm: int = 0, nbr_blocks_per_sm: int = 0):
        """Apply stored launch shapes (ann_set_tuning); zeros restore the built-in rules."""
        t = Tuning()
        for k, g in enumerate(list(tc_groups)[:4]):
            t.tc_groups[k] = int(g)
        t.bp_blocks_per_sm, t.nbr_blocks_per_sm = int(bp_blocks_per_sm), int(nbr_blocks_per_sm)
        self._ck(self.lib.ann_set_tuning(self.h, C.byref(t)))

    # ---- inspection
    def symm_width(self) -> int:
        n = C.c_int32()
        self._ck(self.lib.ann_symm_width(self.h, C.byref(n)))
        return n.value

    def symm(self) -> np.ndarray:
        G = np.zeros((self._last_natoms(), self.symm_width()))
        self._ck(self.lib.ann_get_symm(self.h, _d(G), G.size))
        return G

    def dedg(self) -> np.ndarray:
        G = np.zeros((self._last_natoms(), self.symm_width()))
        self._ck(self.lib.ann_get_dedg(self.h, _d(G), G.size))
        return G

    def atom_energies(self) -> np.ndarray:
        e = np.zeros(self._last_natoms())
        self._ck(self.lib.ann_get_atom_energies(self.h, _d(e), e.size))
        return e

    def _last_natoms(self) -> int:
        return getattr(self, "_N", 0)

    def neighbors(self, with_vectors=False):
        n = C.c_int64()
        self._ck(self.lib.ann_num_neighbors(self.h, C.byref(n)))
        k = n.value
        i = np.zeros(k, np.int32)
        j = np.zeros(k, np.int32)
        img = np.zeros((k, 3), np.int32)
        r = np.zeros((k, 3)) if with_vectors else None
        self._ck(self.lib.ann_get_neighbors(self.h, _i32(i), _i32(j), _i32(img), _d(r), k))
        return i, j, img, r

    # ---- training
    def train_forward(self, offs, posn, types, cell, e_ref, f_ref, w_energy=1.0, w_force=0.1, precision=None):
        prec = self.precision if precision is None else precision
        self._S, self._N = len(offs) - 1, int(offs[-1])
        loss = np.zeros(3)
        self._ck(self.lib.ann_train_forward(self.h, self._S, _i64(np.ascontiguousarray(offs, np.int64)),
                                            _d(np.ascontiguousarray(posn, np.float64)), _i32(np.ascontiguousarray(types, np.int32)),
                                            _d(np.ascontiguousarray(cell, np.float64)), _d(np.ascontiguousarray(e_ref, np.float64)),
                                            _d(np.ascontiguousarray(f_ref, np.float64)), w_energy, w_force, prec, _d(loss)))
        return loss

    def train_forward_staged(self, w_energy=1.0, w_force=0.1, precision=None):
        """The forward pass over the batch and labels of the preceding train_forward, whose neighbour
        rows and symmetry functions stayed on the device (the reference trainer's loop over its
        stored structures): networks, forces, sums and loss with the current parameters."""
        prec = self.precision if precision is None else precision
        loss = np.zeros(3)
        self._ck(self.lib.ann_train_forward_staged(self.h, w_energy, w_force, prec, _d(loss)))
        return loss

    LOSS = {"MSE": 1, "MAE": 2, "HUBER": 3, "ASINH": 4}
    NORM = {"IDENTITY": 0, "LINEAR": 1, "SQRT": 2, "CBRT": 3, "LOG": 4}

    def train_set_loss(self, loss="MSE", norm="LINEAR", delta=1.0):
        """Energy term of the training loss (the reference trainer's LOSS / NORM / DELTA)."""
        lo = self.LOSS[loss] if isinstance(loss, str) else int(loss)
        no = self.NORM[norm] if isinstance(norm, str) else int(norm)
        self._ck(self.lib.ann_train_set_loss(self.h, lo, no, float(delta)))

    def train_backward(self, scale=1.0, download=True):
        """dL/dp (times scale) as an array; download=False leaves the gradient on the device only
        (for adam_step) and returns None."""
        g = np.zeros(self.nparams) if download else None
        self._ck(self.lib.ann_train_backward(self.h, scale, _d(g), self.nparams))
        return g

    def adam_init(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-16):
        """Adam on the device (NN::ADAM; eps defaults to the reference's 1e-16)."""
        self._ck(self.lib.ann_adam_init(self.h, lr, beta1, beta2, eps))

    DECAY = {"CONST": 1, "EXP": 2, "GAUSS": 3, "SQRT": 4, "INV": 5, "STEP": 6}
    REG = {"LASSO": 0, "RIDGE": 1, "HUBER": 2, "ASINH": 3, "NONE": 4}

    OPT = {"SGD": 1, "SDM": 2, "NAG": 3, "ADAGRAD": 4, "ADADELTA": 5, "RMSPROP": 6, "ADAM": 7, "ADAMW": 8, "ADAB": 9, "YOGI": 10,
           "NOGI": 11, "NADAM": 12, "AMSGRAD": 13, "BFGS": 14, "RPROP": 15, "CG": 16}

    def opt_schedule(self, decay="CONST", alpha=0.0, period=1, reg="NONE", eta=0.0):
        """The trainer's step-size schedule (DECAY / ALPHA / PERIOD) and weight decay (REG / ETA)."""
        de = self.DECAY[decay] if isinstance(decay, str) else int(decay)
        rg = self.REG[reg] if isinstance(reg, str) else int(reg)
        self._ck(self.lib.ann_opt_set_schedule(self.h, de, float(alpha), int(period), rg, float(eta)))

    adam_schedule = opt_schedule

    def opt_init(self, algo="ADAM", gamma=1e-3, eta=0.9, eps=1e-8, w=0.0):
        """The trainer's ALGO on the device (opt::algo): step size gamma, momentum / decay eta,
        guard eps, ADAMW weight decay w."""
        a = self.OPT[algo] if isinstance(algo, str) else int(algo)
        self._ck(self.lib.ann_opt_init(self.h, a, float(gamma), float(eta), float(eps), float(w)))

    def opt_step(self, scale=1.0):
        """One optimiser step with the gradient of the last train_backward (times scale)."""
        self._ck(self.lib.ann_opt_step(self.h, scale))

    def adam_step(self, scale=1.0):
        """One Adam step with the gradient of the last train_backward (times scale)."""
        self._ck(self.lib.ann_adam_step(self.h, scale))

    # ---- MD
    def md_init(self, posn, vel, types, cell, masses, dt_fs=2.0, skin=0.5, precision=None):
        prec = self.precision if precision is None else precision
        self._N = len(types)
        self._S = 1
        x = np.ascontiguousarray(posn, np.float64)
        v = np.ascontiguousarray(vel, np.float64)
        t = np.ascontiguousarray(types, np.int32)
        c = np.ascontiguousarray(np.asarray(cell, np.float64).T.reshape(9))
        m = np.ascontiguousarray(masses, np.float64)
        self._ck(self.lib.ann_md_init(self.h, len(t), _d(x), _d(v), _i32(t), _d(c), _d(m), dt_fs, skin, prec))

    def md_run(self, nsteps):
        pe, ke, rb = C.c_double(), C.c_double(), C.c_int32()
        self._ck(self.lib.ann_md_run(self.h, nsteps, C.byref(pe), C.byref(ke), C.byref(rb)))
        return pe.value, ke.value, rb.value

    def network_noalloc(self, natoms: int, type_ptr: int, G_ptr: int, Eatom_ptr: int, dEdG_ptr: int, precision: int = MIXED):
        """ann_network_noalloc on device pointers (integers, e.g. torch tensors' data_ptr())."""
        self._ck(self.lib.ann_network_noalloc(self.h, int(natoms), type_ptr, G_ptr, Eatom_ptr, dEdG_ptr, int(precision)))

    def md_state(self):
        x = np.zeros((self._N, 3))
        v = np.zeros((self._N, 3))
        f = np.zeros((self._N, 3))
        self._ck(self.lib.ann_md_get_state(self.h, _d(x), _d(v), _d(f)))
        return x, v, f
