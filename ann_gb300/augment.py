"""Training-set augmentation of the reference's trainer: Taylor-perturbed copies of structures with
forces (nnptefr2.cpp:2409-2479).

Every structure is kept. One whose mean |F| exceeds 1e-12 gets `nadd` copies in which each atom
j moves by dr_j = vr (sin t cos p, sin t sin p, cos t), with energy E - sum_j dr_j . F_j (the
first-order Taylor estimate) and no forces. cos t and p/pi are std::uniform_real_distribution(-1, 1)
draws; vr comes from the radial distribution (rand/rng.cpp:64-146) with scale rdelta, times the
atom's covalent radius for Perturb::COVALENT. All draws come from one std::mt19937(seed) in the
reference's order (vr, cos t, p per atom), reproduced here bit for bit: MT19937 with the standard
integer seeding, raw 32-bit outputs divided by 2^32 - 1 where the reference divides by gen.max(),
and libstdc++'s generate_canonical<double, 53> (two outputs) for the uniform draws.
"""
from __future__ import annotations

import math

import numpy as np

DIST = {"UNIFORM": 1, "LAPLACE": 2, "NORMAL": 3, "SECH": 5, "LOGISTIC": 6, "COSINE": 7}   # rng::dist::Name values
PI = 3.141592653589793                                                                     # math/const.hpp:9


class _MT:
    def __init__(self, seed: int):
        self.bg = np.random.MT19937(0)
        self.bg._legacy_seeding(seed & 0xFFFFFFFF)
        self.buf, self.k = np.zeros(0, np.uint64), 0

    def raw(self) -> int:
        if self.k == len(self.buf):
            self.buf, self.k = self.bg.random_raw(4096), 0
        v = int(self.buf[self.k])
        self.k += 1
        return v

    def unit(self) -> float:                     # (double)gen() / gen.max()
        return self.raw() / 4294967295.0

    def unit_nonzero(self) -> float:
        p = 0.0
        while p == 0.0:
            p = self.unit()
        return p

    def canonical(self) -> float:                # generate_canonical<double, 53> with a 32-bit engine
        lo = self.raw()
        hi = self.raw()
        u = (lo + hi * 4294967296.0) / 18446744073709551616.0
        return u if u < 1.0 else math.nextafter(1.0, 0.0)


class _Radial:
    def __init__(self, mt: _MT, dist: int, rdelta: float):
        if dist not in DIST.values():
            raise ValueError("Invalid position distribution.")
        self.mt, self.dist, self.s = mt, dist, rdelta
        self.count, self.y = 0, 0.0

    def __call__(self) -> float:
        mt, s = self.mt, self.s
        if self.dist == 1:
            return mt.unit() * s
        if self.dist == 2:
            p = mt.unit_nonzero() - 0.5
            return -1.0 * s * ((p > 0) - (p < 0)) * math.log(1.0 - 2.0 * abs(p))
        if self.dist == 3:
            c = self.count
            self.count += 1
            if c % 2 == 0:
                r1 = mt.unit_nonzero()
                r2 = mt.unit()
                mag = s * math.sqrt(-2.0 * math.log(r1))
                ang = 2.0 * PI * r2
                self.y = mag * math.sin(ang)
                return mag * math.cos(ang)
            return self.y
        p = mt.unit_nonzero()
        if self.dist == 5:
            return s * 2.0 / PI * math.log(math.tan(0.5 * PI * p))
        if self.dist == 6:
            return s * math.log(p / (1.0 - p))
        if p < 0.5:
            t = math.sqrt(-2.0 * math.log(p))
            return s * (0.820251 - 0.806770 * t + 0.093247 * t * t)
        t = math.sqrt(-2.0 * math.log(1.0 - p))
        return -s * (0.820251 - 0.806770 * t + 0.093247 * t * t)


def taylor_perturb(offs, posn, forces, energy, nadd: int, dist="UNIFORM", rdelta: float = 0.05, seed: int = 0, rcov=None):
    """Perturbed training set of packed structures (offs[S+1], posn[N,3], forces[N,3], energy[S]).
    rcov: per-atom covalent radii (Perturb::COVALENT) or None (Perturb::CONSTANT).
    Returns (offs, posn, energy, src): src[k] is the structure each output came from; forces of
    the copies are not defined (the reference clears them)."""
    d = DIST[dist] if isinstance(dist, str) else int(dist)
    mt = _MT(seed)
    radial = _Radial(mt, d, rdelta)
    offs = np.asarray(offs, np.int64)
    posn = np.asarray(posn, np.float64).reshape(-1, 3)
    forces = np.asarray(forces, np.float64).reshape(-1, 3)
    out_x, out_e, out_src, out_n = [], [], [], []
    for s in range(len(offs) - 1):
        a0, a1 = int(offs[s]), int(offs[s + 1])
        n = a1 - a0
        out_x.append(posn[a0:a1]); out_e.append(float(energy[s])); out_src.append(s); out_n.append(n)
        favg = 0.0
        for j in range(a0, a1):
            f = forces[j]
            favg += math.sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2])
        favg /= n
        if not favg > 1.0e-12:
            continue
        for _ in range(nadd):
            xp = posn[a0:a1].copy()
            e = float(energy[s])
            for j in range(n):
                vr = radial()
                if rcov is not None:
                    vr *= float(rcov[a0 + j])
                ct = mt.canonical() * 2.0 - 1.0
                st = math.sqrt(1.0 - ct * ct)
                ph = (mt.canonical() * 2.0 - 1.0) * PI
                dr = (vr * st * math.cos(ph), vr * st * math.sin(ph), vr * ct)
                f = forces[a0 + j]
                xp[j, 0] += dr[0]; xp[j, 1] += dr[1]; xp[j, 2] += dr[2]
                e -= dr[0] * f[0] + dr[1] * f[1] + dr[2] * f[2]
            out_x.append(xp); out_e.append(e); out_src.append(s); out_n.append(n)
    return (np.concatenate([[0], np.cumsum(out_n)]).astype(np.int64), np.concatenate(out_x) if out_x else np.zeros((0, 3)),
            np.array(out_e), np.array(out_src, np.int32))
