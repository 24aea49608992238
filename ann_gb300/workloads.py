"""Seeded synthetic structures and potentials of the five benchmark configurations.

No dataset or checkpoint is used: structures are generated from their stated shapes, sizes and
densities, networks are initialised the way the reference's ANN::resize does (std::mt19937 +
XAVIER-normal, nn.cpp:1071-1190, via ann_init_network), and the input pre-conditioning
(inpb = -mean, inpw = 1/std of the symmetry functions per type) follows the trainer's MEAN/DEV
choice (nnptefr2.cpp:694-871).

Conventions of the reference's basis functions (nnp/basis_radial.cpp:268-272,
basis_angular.cpp:376-381): radial GAUSSIAN exp(-(eta(r-rs))^2) fc(r) with eta in 1/A, so a
textbook eta_B [1/A^2] maps to eta = sqrt(eta_B); angular GAUSS fc fc |1/2+lambda/2 cos|^zeta
exp(-(rij^2+rik^2)/eta^2) with eta a width in A, so eta_B maps to eta = 1/sqrt(eta_B).

Configurations:
  1  Ar FCC 3x3x3 (108 atoms), a=5.26, jitter 0.1 A; rc=6; 8 radial + 8 angular; 16-20-20-1 tanh
  2  256 binary A/B structures, N~U{32..512}, rho=0.05, min distance 1.8 A; rc=6.5;
     12 radial per species + 16 angular per pair = 72; 72-64-64-1 softplus
  3  64 structures as 2 with N~U{32..256}; Lennard-Jones labels (eps 0.0104 eV, sigma 3.4 A, cut 8.5 A)
  4  ternary 1:1:2, 40x40x20 simple-cubic sites (32,000 atoms), a=2.4264 A, jitter 0.15 A; rc=6;
     16 radial per species + 8 angular per pair = 96; 96-128-128-1 tanh
  5  Ar FCC 64x32x32 cells = 262,144 atoms, a=5.26, Maxwell 80 K; configuration-1 basis, 16-32-32-1 tanh;
     for MD the networks carry a Lennard-Jones argon pair potential (lj_argon_text), since
     randomly initialised weights attract atoms without bound
"""
from __future__ import annotations

import math

import numpy as np

SEED0 = 20261203
MASS = {"Ar": 39.948, "A": 39.948, "B": 20.180, "C": 83.798}


# ---------------------------------------------------------------------------------- potentials
def _radial_block(rc: float, eta_b) -> str:
    lines = [f"BasisR COS {rc:f} GAUSSIAN {len(eta_b)}"]
    for e in eta_b:
        lines.append(f"\t{0.0:f} {np.sqrt(e):f}")
    return "\n".join(lines)


def _angular_block(rc: float, eta_b_list, zetas=(1, 2, 4, 8), lambdas=(1, -1)) -> str:
    rows = []
    for eb in eta_b_list:
        for z in zetas:
            for lam in lambdas:
                rows.append((1.0 / np.sqrt(eb), float(z), lam))
    lines = [f"BasisA COS {rc:f} GAUSS {len(rows)}"]
    for e, z, lam in rows:
        lines.append(f"\t{e:f} {z:f} {lam:d} 0")
    return "\n".join(lines)


def potential_text(names, rc, n_radial, ang_eta_b, nodes, neuron, energies=None) -> str:
    """A potential in the reference 'ann' format (NNP::write, nnp.cpp:197-236) with zero networks
    (weights are filled by Context.init_network)."""
    nt = len(names)
    eta_r = np.logspace(np.log10(0.01), np.log10(1.0), n_radial)
    out = ["ann", f"ntypes {nt}"]
    for n in names:
        out.append(f"name {n} mass {MASS.get(n, 1.0):f} energy {(energies or {}).get(n, 0.0):f} ")
    out.append(f"rc {rc:f}")
    for c in names:
        out.append(f"basis {c}")
        for j in names:
            out.append(f"basis_radial {j}")
            out.append(_radial_block(rc, eta_r))
        for a in range(nt):
            for b in range(a, nt):
                out.append(f"basis_angular {names[a]} {names[b]}")
                out.append(_angular_block(rc, ang_eta_b))
    nin = nt * n_radial + (nt * (nt + 1) // 2) * len(ang_eta_b) * 8
    layers = list(nodes)
    for c in names:
        out.append(f"nn {c}")
        out.append("nn " + " ".join(str(x) for x in [nin] + layers) + " ")
        out.append(f"neuron {neuron} 1.000000")
        out.append("inpw " + " ".join(["1.000000000000000"] * nin) + " ")
        out.append("outw 1.000000000000000 ")
        out.append("inpb " + " ".join(["0.000000000000000"] * nin) + " ")
        out.append("outb 0.000000000000000 ")
        prev = nin
        for l, n in enumerate(layers):
            out.append(f"bias[{l + 1}] " + " ".join(["0.000000000000000"] * n) + " ")
        for l, n in enumerate(layers):
            out.append(f"weight[{l},{l + 1}] " + " ".join(["0.000000000000000"] * (n * prev)) + " ")
            prev = n
    return "\n".join(out) + "\n"


CONFIG_POT = {
    1: dict(names=["Ar"], rc=6.0, n_radial=8, ang_eta_b=[0.01], nodes=[20, 20, 1], neuron="TANH"),
    2: dict(names=["A", "B"], rc=6.5, n_radial=12, ang_eta_b=[0.003, 0.01], nodes=[64, 64, 1], neuron="SOFTPLUS"),
    3: dict(names=["A", "B"], rc=6.5, n_radial=12, ang_eta_b=[0.003, 0.01], nodes=[64, 64, 1], neuron="SOFTPLUS"),
    4: dict(names=["A", "B", "C"], rc=6.0, n_radial=16, ang_eta_b=[0.01], nodes=[128, 128, 1], neuron="TANH"),
    5: dict(names=["Ar"], rc=6.0, n_radial=8, ang_eta_b=[0.01], nodes=[32, 32, 1], neuron="TANH"),
}


def config_potential_text(cfg: int, seed: int | None = None, with_weights: bool = True) -> str:
    """The configuration's potential text; with_weights draws every network as ANN::resize does
    (std::mt19937(seed + 1000*type), XAVIER normal, sigma_w=1, sigma_b=0.001) in pure Python, so
    that no GPU is needed to produce it (identical to Context.init_network)."""
    spec = CONFIG_POT[cfg]
    text = potential_text(**spec)
    if not with_weights:
        return text
    s0 = SEED0 + cfg if seed is None else seed
    nt = len(spec["names"])
    nin = nt * spec["n_radial"] + (nt * (nt + 1) // 2) * len(spec["ang_eta_b"]) * 8
    nodes = spec["nodes"]
    params = [xavier_network(s0 + 1000 * t, nin, nodes) for t in range(nt)]
    return set_network_text(text, params, nin, nodes)


class _StdMT19937Normal:
    """std::mt19937 + std::normal_distribution<double> of libstdc++ (Marsaglia polar method with
    one cached value; uniform draws by generate_canonical<double,53>: two 32-bit outputs)."""

    def __init__(self, seed: int):
        bg = np.random.MT19937(0)
        bg._legacy_seeding(seed & 0xFFFFFFFF)   # init_genrand(seed), as std::mt19937(seed)
        self.bg = bg
        self.saved = None

    def reset(self):                              # a fresh distribution object drops the cache
        self.saved = None

    def _u(self) -> float:
        lo, hi = (int(v) for v in self.bg.random_raw(2))
        u = (lo + hi * 4294967296.0) / 18446744073709551616.0
        return u if u < 1.0 else float(np.nextafter(1.0, 0.0))

    def normal(self, sd: float) -> float:
        if self.saved is not None:
            v, self.saved = self.saved, None
            return v * sd
        while True:
            x = 2.0 * self._u() - 1.0
            y = 2.0 * self._u() - 1.0
            r2 = x * x + y * y
            if r2 <= 1.0 and r2 != 0.0:
                break
        mult = math.sqrt(-2.0 * math.log(r2) / r2)   # libm, as std::log / std::sqrt
        self.saved = x * mult
        return y * mult * sd


def xavier_network(seed: int, nin: int, nodes, sigma_b: float = 0.001, sigma_w: float = 1.0):
    """Biases then weights of one network in the reference packing (nn.cpp:846-859, weights
    column-major), drawn exactly as ANN::resize with dist NORMAL and init XAVIER (nn.cpp:1071-1190)."""
    g = _StdMT19937Normal(seed)
    ni = [nin] + list(nodes[:-1])
    out = []
    for l, no in enumerate(nodes):
        g.reset()
        s = sigma_b * np.sqrt(2.0 / (no + ni[l]))
        out.extend(g.normal(s) for _ in range(no))
    for l, no in enumerate(nodes):
        g.reset()
        s = sigma_w * np.sqrt(2.0 / (no + ni[l]))
        out.extend(g.normal(s) for _ in range(no * ni[l]))
    return np.array(out)


def set_network_text(text: str, params, nin: int, nodes) -> str:
    """Replace the bias/weight rows of each 'nn' block (types in file order) by packed parameters."""
    lines = text.splitlines()
    ni = [nin] + list(nodes[:-1])
    t = -1
    out = []
    for ln in lines:
        tok = ln.split()
        if len(tok) == 2 and tok[0] == "nn":
            t += 1
        if tok and (tok[0].startswith("bias[") or tok[0].startswith("weight[")):
            p = params[t]
            if tok[0].startswith("bias["):
                l = int(tok[0][5:-1]) - 1
                off = sum(nodes[:l])
                vals = p[off:off + nodes[l]]
            else:
                l = int(tok[0][7:].split(",")[0])
                off = sum(nodes) + sum(nodes[q] * ni[q] for q in range(l))
                vals = p[off:off + nodes[l] * ni[l]].reshape(ni[l], nodes[l]).T.reshape(-1)   # file rows: row-major
            ln = tok[0] + " " + " ".join(f"{v:.15f}" for v in vals) + " "
        out.append(ln)
    return "\n".join(out) + "\n"


def make_potential(ctx, cfg: int, seed: int | None = None):
    """Load the configuration's potential into ctx and initialise its networks on the library side
    (ann_init_network: Xavier normal, sigma_w=1, sigma_b=0.001, the ANNP defaults nn.cpp:1589-1590)
    with per-type seeds seed+1000*type."""
    ctx.load_text(config_potential_text(cfg, with_weights=False))
    s0 = SEED0 + cfg if seed is None else seed
    for t in range(ctx.ntypes):
        ctx.init_network(t, s0 + 1000 * t, dist=0, init=4, sigma_b=0.001, sigma_w=1.0)
    return ctx


def precondition(ctx, offs, posn, types, cell, symm=None):
    """inpb = -mean(G), inpw = 1/std(G) per type from the FP64 symmetry functions of a batch
    (PreBias::MEAN, PreScale::DEV, nnptefr2.cpp:771-849)."""
    from . import FP64
    if symm is None:
        ctx.compute(offs, posn, types, cell, forces=False, virial=False, precision=FP64)
        symm = ctx.symm()
    for t in range(ctx.ntypes):
        nin = ctx.num_inputs(t)
        G = symm[types == t, :nin]
        if len(G) < 2:
            continue
        mu = G.mean(axis=0)
        sd = G.std(axis=0, ddof=1)
        w = np.where(sd > 0, 1.0 / np.where(sd > 0, sd, 1.0), 1.0)
        ctx.set_input_scaling(t, w, -mu)


# ------------------------------------------------------------ a pair potential held by a network
def radial_eta(n_radial: int) -> np.ndarray:
    """The radial widths potential_text writes (eta = sqrt(eta_B), eta_B log-spaced 0.01..1 A^-2),
    rounded as they are printed, so that host-side sums match the loaded potential."""
    return np.array([float(f"{np.sqrt(e):f}") for e in np.logspace(np.log10(0.01), np.log10(1.0), n_radial)])


def _radial_g(r, rc, eta):
    """GAUSSIAN radial functions with rs = 0 and the COS cutoff, g_i(r) = exp(-(eta_i r)^2) fc(r),
    and their r-derivatives (basis_radial.cpp:268-272, cutoff.hpp COS)."""
    r = np.asarray(r, float)[:, None]
    inside = r < rc
    fc = np.where(inside, 0.5 * (np.cos(np.pi * r / rc) + 1.0), 0.0)
    dfc = np.where(inside, -0.5 * np.pi / rc * np.sin(np.pi * r / rc), 0.0)
    e = np.exp(-(eta[None, :] * r) ** 2)
    return e * fc, e * (-2.0 * eta[None, :] ** 2 * r * fc + dfc)


def lj_pair_coefficients(rc, eta, eps=0.0104, sig=3.405, r0=3.0, lam=1e-8):
    """c such that phi(r) = 2 c.g(r) follows the Lennard-Jones pair energy shifted to zero at rc
    (argon: eps 10.4 meV, sigma 3.405 A) on [r0, rc]: ridge-regularised least squares on values and
    derivatives, weighted towards the first-neighbour shell. A network whose atomic energy is c.G
    then carries phi as its pair potential, since sum_atoms c.G_atom = sum_pairs 2 c.g(r)."""
    r = np.linspace(r0, rc, 400)
    g, dg = _radial_g(r, rc, eta)
    u = (sig / r) ** 6
    phi = 4.0 * eps * u * (u - 1.0) - 4.0 * eps * ((sig / rc) ** 6) * ((sig / rc) ** 6 - 1.0)
    dphi = -24.0 * eps * u * (2.0 * u - 1.0) / r
    w = np.tile(np.exp(-0.5 * (r - 3.8) ** 2) + 0.05, 2)
    A = np.vstack([g, 0.3 * dg]) * w[:, None]
    b = np.concatenate([phi, 0.3 * dphi]) / 2.0 * w
    return np.linalg.solve(A.T @ A + lam * np.eye(len(eta)), A.T @ b)


def fcc_radial_sums(a, rc, eta) -> np.ndarray:
    """Per-atom radial symmetry functions G_i = sum_j g_i(r_j) of a perfect FCC crystal."""
    n = int(np.ceil(rc / a)) + 1
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(*[np.arange(-n, n + 1)] * 3, indexing="ij"), -1).reshape(-1, 3)
    d = np.linalg.norm(((g[:, None, :] + basis[None]).reshape(-1, 3)) * a, axis=1)
    d = d[(d > 1e-9) & (d < rc)]
    return _radial_g(d, rc, eta)[0].sum(axis=0)


def linear_network(coef, nin: int, nodes, seed: int, scale: float = 0.003, out_bias: float = 0.0):
    """Packed parameters (reference packing, nn.cpp:846-859) of a tanh network whose output is
    coef.z + out_bias to a relative 1e-5 over |coef.z| <= 1: the first layer writes scale*u_k*(coef.z)
    into every unit (u ~ N(0,1)), the second mixes them with N(0,1/32) weights, and the output
    weights are rescaled so the small-signal gain is one. Every unit is active, so the network
    costs what a trained one does."""
    rng = np.random.default_rng(seed)
    coef = np.asarray(coef, float)
    h1, h2 = nodes[0], nodes[1]
    u = rng.normal(0.0, 1.0, h1)
    W1 = scale * np.outer(np.pad(coef, (0, nin - len(coef))), u)           # [in, out]
    W2 = rng.normal(0.0, 1.0 / np.sqrt(h1), (h1, h2))
    w3 = rng.normal(0.0, 1.0 / np.sqrt(h2), h2)
    gain = scale * float(u @ W2 @ w3)
    if abs(gain) < 1e-6 * scale:
        raise ValueError("degenerate draw for the linear network: choose another seed")
    w3 /= gain
    biases = np.concatenate([np.zeros(h1), np.zeros(h2), [out_bias]])
    return np.concatenate([biases, W1.reshape(-1), W2.reshape(-1), w3])


def lj_argon_text(cfg: int = 5, a: float = 5.26, seed: int | None = None) -> str:
    """The configuration's potential (one type, tanh networks) with weights that make it the
    Lennard-Jones argon pair potential of lj_pair_coefficients: radial inputs shifted by their FCC
    values at lattice constant a (inpb = -G(a), so c.z stays small and free of cancellation), the
    angular inputs weighted zero, and c.G(a) as the output bias. Unlike randomly initialised
    weights, which attract atoms without bound, this keeps an FCC crystal stable under MD."""
    spec = CONFIG_POT[cfg]
    if len(spec["names"]) != 1 or spec["neuron"] != "TANH" or len(spec["nodes"]) != 3:
        raise ValueError("lj_argon_text needs a one-type configuration with two tanh hidden layers")
    rc, nr = spec["rc"], spec["n_radial"]
    eta = radial_eta(nr)
    c = lj_pair_coefficients(rc, eta)
    G0 = fcc_radial_sums(a, rc, eta)
    nin = nr + len(spec["ang_eta_b"]) * 8
    p = linear_network(c, nin, spec["nodes"], SEED0 + cfg if seed is None else seed, out_bias=float(c @ G0))
    text = set_network_text(potential_text(**spec), [p], nin, spec["nodes"])
    inpb = np.concatenate([-G0, np.zeros(nin - nr)])
    return "\n".join(("inpb " + " ".join(f"{v:.15f}" for v in inpb) + " ") if ln.startswith("inpb ") else ln
                     for ln in text.splitlines()) + "\n"


# ---------------------------------------------------------------------------------- structures
def fcc(nx, ny, nz, a):
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    x = (g[:, None, :] + basis[None, :, :]).reshape(-1, 3) * a
    R = np.diag([nx * a, ny * a, nz * a])
    return x, R


def config1(seed: int = SEED0 + 1):
    rng = np.random.default_rng(seed)
    x, R = fcc(3, 3, 3, 5.26)
    x = x + rng.normal(0.0, 0.1, x.shape)
    return [(x, np.zeros(len(x), np.int32), R)]


def _rsa(rng, n, L, dmin, max_tries=200000):
    x = np.zeros((n, 3))
    k = 0
    tries = 0
    d2 = dmin * dmin
    while k < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("random sequential addition did not converge")
        p = rng.uniform(0.0, L, 3)
        if k:
            d = x[:k] - p
            d -= L * np.round(d / L)
            if np.min(np.einsum("ij,ij->i", d, d)) < d2:
                continue
        x[k] = p
        k += 1
    return x


def random_binary(nstruc, nmin, nmax, rho=0.05, dmin=1.8, seed=SEED0 + 2):
    """Binary structures: N~U{nmin..nmax}, floor(N/2) of type 0 and the rest type 1 in shuffled
    order, cubic box L=(N/rho)^(1/3), random sequential addition with minimum-image distance >= dmin."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nstruc):
        n = int(rng.integers(nmin, nmax + 1))
        L = (n / rho) ** (1.0 / 3.0)
        x = _rsa(rng, n, L, dmin)
        t = np.array([0] * (n // 2) + [1] * (n - n // 2), np.int32)
        rng.shuffle(t)
        out.append((x, t, np.eye(3) * L))
    return out


def config2(seed: int = SEED0 + 2, nstruc: int = 256):
    return random_binary(nstruc, 32, 512, seed=seed)


def config3(seed: int = SEED0 + 3, nstruc: int = 64):
    return random_binary(nstruc, 32, 256, seed=seed)


def config4(seed: int = SEED0 + 4, dims=(40, 40, 20)):
    rng = np.random.default_rng(seed)
    a = (1.0 / 0.07) ** (1.0 / 3.0)
    g = np.stack(np.meshgrid(*[np.arange(d) for d in dims], indexing="ij"), -1).reshape(-1, 3).astype(np.float64)
    x = g * a + rng.normal(0.0, 0.15, g.shape)
    n = len(x)
    t = np.array([0] * (n // 4) + [1] * (n // 4) + [2] * (n - 2 * (n // 4)), np.int32)
    rng.shuffle(t)
    return [(x, t, np.diag([d * a for d in dims]))]


def config5(seed: int = SEED0 + 5, cells=(64, 32, 32), T=80.0):
    """FCC Ar box and Maxwell-Boltzmann velocities (A/fs) with zero net momentum."""
    rng = np.random.default_rng(seed)
    x, R = fcc(*cells, 5.26)
    m = MASS["Ar"]
    kb = 8.617333262e-5          # eV/K (chem/units.cpp:149)
    mvv = 103.642696526805       # eV per Da A^2/fs^2 (chem/units.cpp:151)
    sig = np.sqrt(kb * T / (m * mvv))
    v = rng.normal(0.0, sig, x.shape)
    v -= v.mean(axis=0)
    return x, v, np.zeros(len(x), np.int32), R


def ghost_domain(x, types, R, rcomm):
    """What an MD engine (LAMMPS, one domain, newton_pair on) passes a pair style for a periodic
    structure: local atoms (x wrapped into the cell R, lattice vectors as columns) followed by ghost
    atoms (images x_j + R n, n != 0, inside the cell padded by rcomm on every face) and a FULL
    neighbour list of every local atom within rcomm (self excluded). Returns (x_all, type_all,
    owner, numneigh, neigh); rows are in increasing neighbour index."""
    from scipy.spatial import cKDTree
    R = np.asarray(R, np.float64)
    Ri = np.linalg.inv(R)
    s = np.asarray(x, np.float64) @ Ri.T
    s -= np.floor(s)
    s[s >= 1.0] = 0.0
    xl = s @ R.T
    n = len(xl)
    vol = abs(np.linalg.det(R))
    h = np.array([vol / np.linalg.norm(np.cross(R[:, (d + 1) % 3], R[:, (d + 2) % 3])) for d in range(3)])
    pad = rcomm / h
    k = np.ceil(pad).astype(int)
    gx, go = [xl], [np.arange(n)]
    for n0 in range(-k[0], k[0] + 1):
        for n1 in range(-k[1], k[1] + 1):
            for n2 in range(-k[2], k[2] + 1):
                if n0 == n1 == n2 == 0:
                    continue
                sn = s + np.array([n0, n1, n2], np.float64)
                keep = np.all((sn > -pad) & (sn < 1.0 + pad), axis=1)
                if keep.any():
                    gx.append(xl[keep] + R @ np.array([n0, n1, n2], np.float64))
                    go.append(np.nonzero(keep)[0])
    X = np.concatenate(gx)
    owner = np.concatenate(go).astype(np.int64)
    T = np.asarray(types, np.int32)[owner]
    pairs = cKDTree(X).query_pairs(rcomm, output_type="ndarray")
    a, b = pairs[:, 0], pairs[:, 1]
    strict = np.einsum("ij,ij->i", X[a] - X[b], X[a] - X[b]) < rcomm * rcomm    # |r| < rcomm, as the list builders
    a, b = a[strict], b[strict]
    src = np.concatenate([a[a < n], b[b < n]])
    dst = np.concatenate([b[a < n], a[b < n]])
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    numneigh = np.bincount(src, minlength=n).astype(np.int32)
    return X, T, owner, numneigh, dst.astype(np.int32)


def lennard_jones(structures, eps=0.0104, sig=3.4, rcut=8.5):
    """Unshifted, truncated LJ energies and forces (pot_lj_cut.cpp:73-90: 1/2 sum over the full
    periodic-image list) for synthetic training labels."""
    E = []
    F = []
    for x, t, R in structures:
        Ri = np.linalg.inv(R)
        n = len(x)
        s = x @ Ri.T
        gn = np.linalg.norm(Ri, axis=1)
        ds = s[:, None, :] - s[None, :, :]
        e = 0.0
        f = np.zeros_like(x)
        lo = np.floor(ds.min(axis=(0, 1)) - rcut * gn).astype(int) - 1
        hi = np.ceil(ds.max(axis=(0, 1)) + rcut * gn).astype(int) + 1
        for n0 in range(lo[0], hi[0] + 1):
            for n1 in range(lo[1], hi[1] + 1):
                for n2 in range(lo[2], hi[2] + 1):
                    shift = R @ np.array([n0, n1, n2], float)
                    r = x[:, None, :] - x[None, :, :] - shift
                    d2 = np.einsum("ijk,ijk->ij", r, r)
                    if n0 == 0 and n1 == 0 and n2 == 0:
                        np.fill_diagonal(d2, np.inf)
                    m = d2 < rcut * rcut
                    if not m.any():
                        continue
                    d = np.sqrt(np.where(m, d2, 1.0))
                    du6 = np.where(m, (sig / d) ** 6, 0.0)
                    e += 0.5 * np.sum(4.0 * eps * du6 * (du6 - 1.0))
                    fmag = np.where(m, 24.0 * eps * du6 * (2.0 * du6 - 1.0) / (d * d), 0.0)
                    f += np.einsum("ij,ijk->ik", fmag, r)
        E.append(e)
        F.append(f)
    return np.array(E), F
