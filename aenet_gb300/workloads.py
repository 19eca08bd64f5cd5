"""Seeded synthetic structures and random-weight potentials.

Five workloads, one per evaluated configuration:

  cu_fcc_256        Cu FCC 4x4x4 conventional cells (256 atoms), a = 3.61,
                    N(0, 0.05) displacements; Chebyshev radial order 16
                    (Rc 6.0) / angular order 8 (Rc 4.0): 26 features;
                    26-20-20-1 network.
  aucu_fcc_4000     Au/Cu 50/50 FCC 10x10x10 (4000 atoms), a = 3.90,
                    N(0, 0.08); Chebyshev 12 (6.5) / 6 (4.5), species-typed:
                    40 features; 40-25-25-1 per species.
  tio2_rutile_9000  rutile Ti/O 10x10x15 unit cells (9000 atoms), a = 4.59,
                    c = 2.96, u = 0.305, N(0, 0.1); Behler G2 (8 eta per
                    pair, log-spaced 0.003-0.5, Rs = 0) and G4 (zeta 1, 2, 4,
                    16 x lambda +-1 x eta 0.003, 0.03 per triple), Rc = 6.5:
                    64 features; 64-30-30-1 per species.
  lisio_batch_4096  4096 cubic Li/Si/O cells, atom counts log-uniform in
                    [16, 512], density 0.08 / A^3, random sequential
                    placement with 1.6 A minimum separation, fractions
                    0.3/0.3/0.4; Chebyshev 10 (6.0) / 4 (4.0): 32 features;
                    32-32-32-1 per species.
  cuau_fcc_1m       Cu/Au (25% Au) FCC 64^3 conventional cells (1,048,576
                    atoms), a = 3.70, N(0, 0.1); Chebyshev 16 (6.0) / 8 (4.0),
                    species-typed: 52 features; 52-20-20-1 per species.

Random streams (numpy default_rng(seed)) are drawn in a fixed order:
species assignment (exact-count permutation), positions/displacements,
network weights per species in type order (Glorot-uniform over the full
n_out x (n_in + 1) matrix, bias column included), velocities.  Potential
files carry TrnSet info scale 0.5, shift -3.0, E_atom(k) = -k eV for the
k-th species, Rc_min 1.5 A, environment order = type order; their
normalisation statistics are the running statistics of stp_eval
(sfsetup.f90:960-975) over the workload's own atoms, computed by a
caller-supplied descriptor function.
"""
import os

import numpy as np

from . import nnfile

RC_MIN = 1.5
TS_SCALE = 0.5
TS_SHIFT = -3.0
MASSES = {"Cu": 63.546, "Au": 196.96657, "Li": 6.94, "Si": 28.085, "O": 15.999, "Ti": 47.867}


class Structure:
    def __init__(self, positions, types, cell, pbc=True):
        self.positions = np.ascontiguousarray(positions, dtype=np.float64)
        self.types = np.ascontiguousarray(types, dtype=np.int32)   # 1-based
        self.cell = np.ascontiguousarray(cell, dtype=np.float64)
        self.pbc = bool(pbc)

    @property
    def natoms(self):
        return self.positions.shape[0]


class Workload:
    def __init__(self, name, types, setups, arch, structures, seed):
        self.name = name
        self.types = list(types)
        self.setups = setups            # species -> Setup dict
        self.arch = arch
        self.structures = structures
        self.seed = seed
        self.networks = None
        self.velocities = None

    @property
    def natoms(self):
        return int(sum(s.natoms for s in self.structures))

    def packed(self):
        """(natoms per structure, positions, types, cells, pbc) packed."""
        nat = np.array([s.natoms for s in self.structures], dtype=np.int32)
        pos = np.concatenate([s.positions for s in self.structures])
        typ = np.concatenate([s.types for s in self.structures]).astype(np.int32)
        cells = np.stack([s.cell for s in self.structures])
        pbc = np.array([int(s.pbc) for s in self.structures], dtype=np.int32)
        return nat, pos, typ, cells, pbc


def glorot_networks(rng, types, arch):
    nets = {}
    for t in types:
        W = []
        for l in range(len(arch) - 1):
            nin, nout = arch[l], arch[l + 1]
            lim = np.sqrt(6.0 / ((nin + 1) + nout))
            M = rng.uniform(-lim, lim, size=(nout, nin + 1))
            W.append(M.ravel(order="F"))        # Fortran column-major slice
        nets[t] = nnfile.make_network(arch, np.concatenate(W))
    return nets


def fcc_positions(n, a):
    basis = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    g = np.arange(n)
    cells = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    pos = (cells[:, None, :] + basis[None, :, :]).reshape(-1, 3) * a
    return pos, np.eye(3) * (n * a)


def exact_species(rng, n, fractions):
    counts = [int(round(f * n)) for f in fractions[:-1]]
    counts.append(n - sum(counts))
    lab = np.concatenate([np.full(c, k + 1, dtype=np.int32) for k, c in enumerate(counts)])
    return lab[rng.permutation(n)]


def cheb_setups(types, r_order, r_Rc, a_order, a_Rc):
    return {t: nnfile.chebyshev_setup(t, types, r_Rc, r_order, a_Rc, a_order, RC_MIN)
            for t in types}


def cu_fcc_256(seed=1):
    rng = np.random.default_rng(seed)
    types = ["Cu"]
    pos, cell = fcc_positions(4, 3.61)
    species = exact_species(rng, len(pos), [1.0])
    pos = pos + rng.normal(0.0, 0.05, pos.shape)
    arch = [26, 20, 20, 1]
    w = Workload("cu_fcc_256", types, cheb_setups(types, 16, 6.0, 8, 4.0), arch,
                 [Structure(pos, species, cell)], seed)
    w.networks = glorot_networks(rng, types, arch)
    return w


def aucu_fcc_4000(seed=2):
    rng = np.random.default_rng(seed)
    types = ["Au", "Cu"]
    pos, cell = fcc_positions(10, 3.90)
    species = exact_species(rng, len(pos), [0.5, 0.5])
    pos = pos + rng.normal(0.0, 0.08, pos.shape)
    arch = [40, 25, 25, 1]
    w = Workload("aucu_fcc_4000", types, cheb_setups(types, 12, 6.5, 6, 4.5), arch,
                 [Structure(pos, species, cell)], seed)
    w.networks = glorot_networks(rng, types, arch)
    return w


def rutile_positions(nx, ny, nz, a, c, u):
    frac = np.array([[0, 0, 0], [.5, .5, .5], [u, u, 0], [-u, -u, 0],
                     [.5 + u, .5 - u, .5], [.5 - u, .5 + u, .5]])
    spec = np.array([1, 1, 2, 2, 2, 2], dtype=np.int32)
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"),
                 -1).reshape(-1, 3)
    f = (g[:, None, :] + frac[None, :, :]).reshape(-1, 3)
    scale = np.array([a, a, c])
    pos = f * scale
    species = np.tile(spec, len(g))
    cell = np.diag([nx * a, ny * a, nz * c])
    return pos, species, cell


def behler_functions(types, rc=6.5):
    """8 G2 per pair, 16 G4 per triple (file order: all G2 then all G4)."""
    funcs = []
    etas2 = np.geomspace(0.003, 0.5, 8)
    for t2 in types:
        for eta in etas2:
            funcs.append({"G": 2, "type2": t2, "Rc": rc, "Rs": 0.0, "eta": float(eta)})
    for i, t2 in enumerate(types):
        for t3 in types[i:]:
            for zeta in (1.0, 2.0, 4.0, 16.0):
                for lam in (1.0, -1.0):
                    for eta in (0.003, 0.03):
                        funcs.append({"G": 4, "type2": t2, "type3": t3, "Rc": rc,
                                      "lambda": lam, "zeta": zeta, "eta": eta})
    return funcs


def tio2_rutile_9000(seed=3, cells=(10, 10, 15)):
    rng = np.random.default_rng(seed)
    types = ["Ti", "O"]
    pos, species, cell = rutile_positions(cells[0], cells[1], cells[2], 4.59, 2.96, 0.305)
    pos = pos + rng.normal(0.0, 0.1, pos.shape)
    funcs = behler_functions(types)
    setups = {t: nnfile.behler_setup(t, types, funcs, RC_MIN) for t in types}
    arch = [len(funcs), 30, 30, 1]
    w = Workload("tio2_rutile_9000", types, setups, arch, [Structure(pos, species, cell)], seed)
    w.networks = glorot_networks(rng, types, arch)
    return w


def random_cell(rng, n, density=0.08, dmin=1.6, max_tries=200000):
    L = (n / density) ** (1.0 / 3.0)
    pts = np.empty((n, 3))
    k = tries = 0
    d2 = dmin * dmin
    while k < n:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("random placement failed")
        p = rng.uniform(0.0, L, 3)
        if k:
            d = pts[:k] - p
            d -= L * np.round(d / L)
            if np.min(np.einsum("ij,ij->i", d, d)) < d2:
                continue
        pts[k] = p
        k += 1
    return pts, np.eye(3) * L


def lisio_batch_4096(seed=4, nstruc=4096):
    rng = np.random.default_rng(seed)
    types = ["Li", "Si", "O"]
    sizes = np.rint(np.exp(rng.uniform(np.log(16), np.log(512), nstruc))).astype(int)
    structs = []
    for n in sizes:
        species = exact_species(rng, int(n), [0.3, 0.3, 0.4])
        pos, cell = random_cell(rng, int(n))
        structs.append(Structure(pos, species, cell))
    arch = [32, 32, 32, 1]
    w = Workload("lisio_batch_4096", types, cheb_setups(types, 10, 6.0, 4, 4.0), arch,
                 structs, seed)
    w.networks = glorot_networks(rng, types, arch)
    return w


def cuau_fcc_1m(seed=5, n=64):
    rng = np.random.default_rng(seed)
    types = ["Cu", "Au"]
    pos, cell = fcc_positions(n, 3.70)
    species = exact_species(rng, len(pos), [0.75, 0.25])
    pos = pos + rng.normal(0.0, 0.1, pos.shape)
    arch = [52, 20, 20, 1]
    w = Workload("cuau_fcc_1m", types, cheb_setups(types, 16, 6.0, 8, 4.0), arch,
                 [Structure(pos, species, cell)], seed)
    w.networks = glorot_networks(rng, types, arch)
    # Maxwell-Boltzmann velocities at 600 K (A/fs), centre of mass removed
    from .md import maxwell_boltzmann
    v = maxwell_boltzmann([MASSES[types[t - 1]] for t in species], 600.0, rng)
    w.velocities = v
    return w


WORKLOADS = {f.__name__: f for f in (cu_fcc_256, aucu_fcc_4000, tio2_rutile_9000,
                                     lisio_batch_4096, cuau_fcc_1m)}


def running_stats(vecs):
    """stp_eval's running min/max/avg/cov (sfsetup.f90:960-975)."""
    vecs = np.asarray(vecs, dtype=np.float64)
    mn, mx, av, cv = vecs[0].copy(), vecs[0].copy(), vecs[0].copy(), vecs[0] * vecs[0]
    for e in range(1, vecs.shape[0]):
        v = vecs[e]
        mn = np.minimum(mn, v)
        mx = np.maximum(mx, v)
        av = (e * av + v) / (e + 1)
        cv = (e * cv + v * v) / (e + 1)
    return mn, mx, av, cv


def write_potentials(workload, directory, descriptor_fn=None, stats=None, networks=None,
                     max_atoms_for_stats=20000):
    """Write one .nn per species and return {species: path}.

    ``descriptor_fn(workload, paths, atom_ids)`` must return raw
    (unnormalised) descriptors of the given atoms as an (n, nsf) array and
    their species; it is called with identity-normalisation potentials.
    ``stats`` (species -> (min, max, avg, cov)) skips that step.
    """
    os.makedirs(directory, exist_ok=True)
    nets = networks or workload.networks
    types = workload.types
    ts = {"scale": TS_SCALE, "shift": TS_SHIFT, "typeName": types,
          "E_atom": [-float(k + 1) for k in range(len(types))]}

    def dump(stat_map, tag):
        paths = {}
        for t in types:
            stp = dict(workload.setups[t])
            mn, mx, av, cv = stat_map[t]
            stp["sfval_min"], stp["sfval_max"], stp["sfval_avg"], stp["sfval_cov"] = mn, mx, av, cv
            p = os.path.join(directory, "%s%s.nn" % (t, tag))
            nnfile.write_nn(p, nets[t], stp, ts)
            paths[t] = p
        return paths

    if stats is None:
        ident = {}
        for t in types:
            nsf = workload.setups[t]["nsf"]
            ident[t] = (np.zeros(nsf), np.zeros(nsf), np.zeros(nsf), np.ones(nsf))
        ipaths = dump(ident, ".identity")
        nat = workload.natoms
        ids = np.arange(nat) if nat <= max_atoms_for_stats else np.sort(
            np.random.default_rng(workload.seed + 1000).choice(nat, max_atoms_for_stats,
                                                               replace=False))
        G, spec = descriptor_fn(workload, ipaths, ids)
        stats = {}
        for k, t in enumerate(types, start=1):
            sel = G[spec == k]
            if sel.shape[0] == 0:
                nsf = workload.setups[t]["nsf"]
                stats[t] = (np.zeros(nsf), np.zeros(nsf), np.zeros(nsf), np.ones(nsf))
            else:
                stats[t] = running_stats(sel)
    return dump(stats, "")


def gpu_descriptor_fn(workload, paths, ids):
    """Raw descriptors of the selected atoms from the FP64 GPU path
    (identity-normalisation potentials), for :func:`write_potentials`."""
    import torch
    from .core import ANNPotentials, FP64
    from .plan import Plan
    ann = ANNPotentials({t: paths[t] for t in workload.types})
    try:
        nat, pos, typ, cells, pbc = workload.packed()
        plan = Plan(nat, cells, pbc, precision=FP64, coords0=pos)
        p = torch.tensor(pos, device="cuda")
        t = torch.tensor(typ, device="cuda")
        plan.forward(p, t)
        plan.check()
        G = plan.descriptors()
        ids_t = torch.as_tensor(np.asarray(ids), device="cuda").long()
        rows = G[ids_t].cpu().numpy()
        nsf = max(workload.setups[s]["nsf"] for s in workload.types)
        plan.close()
    finally:
        ann.release()
    return rows[:, :nsf], typ[np.asarray(ids)]
