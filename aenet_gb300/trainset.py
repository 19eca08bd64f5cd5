"""aenet training-set files (TrnSet, the binary records of src/trainset.f90).

Layout (Fortran unformatted sequential records, little endian):
  header    nTypes | nStrucs | typeName(2*nTypes chars) | E_atom(nTypes) f8 |
            normalized (logical4) | scale f8 | shift f8          (ts_write_header)
  structure len_trim(filename) | filename | nAtoms, nTypes | energy f8
            per atom: itype | cooCart(3) f8 | forCart(3) f8 | nsf | sfval(nsf) f8
            (ts_write_structure_info / ts_write_atom_info / ts_write_sf_info)
  footer    nAtomsTot | E_av, E_min, E_max | has_setups (logical4) |
            per type: itype, then the Setup records of a potential file
            (ts_write_footer, save_Setup)

:func:`normalize` restates ts_normalize (src/trainset.f90:1160-1271 with
ts_energy_norm_simple, 1275-1295): energies to scale (E - N shift) with
scale = 2/(E_max - E_min), shift = (E_max + E_min)/2 (per atom), forces
times scale, descriptors normalised with the footer setups' statistics.
"""
import struct

import numpy as np

__all__ = ["TrainSet", "read_trainset", "write_trainset", "normalize"]


class TrainSet:
    def __init__(self, type_names, E_atom, normalized=False, scale=1.0, shift=0.0):
        self.type_names = list(type_names)
        self.E_atom = np.asarray(E_atom, dtype=np.float64)
        self.normalized = bool(normalized)
        self.scale = float(scale)
        self.shift = float(shift)
        self.structures = []     # dicts: file, energy, types (1-based), coords, forces, sfval
        self.setup_records = None   # per type: list of raw Setup records, or None
        self.E_av = self.E_min = self.E_max = 0.0

    @property
    def natoms_total(self):
        return int(sum(len(s["types"]) for s in self.structures))

    def add(self, filename, energy, types, coords, forces, sfval):
        self.structures.append({"file": str(filename), "energy": float(energy),
                                "types": np.asarray(types, dtype=np.int32),
                                "coords": np.asarray(coords, dtype=np.float64).reshape(-1, 3),
                                "forces": np.asarray(forces, dtype=np.float64).reshape(-1, 3),
                                "sfval": [np.asarray(v, dtype=np.float64) for v in sfval]})

    def energy_range(self):
        """Per-atom E_av, E_min, E_max over the structures."""
        e = np.array([s["energy"] / len(s["types"]) for s in self.structures])
        return float(e.mean()), float(e.min()), float(e.max())


def _records(data):
    recs, i = [], 0
    while i < len(data):
        (n,) = struct.unpack_from("<i", data, i)
        (m,) = struct.unpack_from("<i", data, i + 4 + n)
        if m != n:
            raise ValueError("corrupt record framing")
        recs.append(data[i + 4:i + 4 + n])
        i += 8 + n
    return recs


def _rec(payload):
    return struct.pack("<i", len(payload)) + payload + struct.pack("<i", len(payload))


def read_trainset(path):
    recs = _records(open(path, "rb").read())
    it = iter(recs)
    i4 = lambda r: np.frombuffer(r, "<i4")
    f8 = lambda r: np.frombuffer(r, "<f8")
    ntypes = int(i4(next(it))[0])
    nstrucs = int(i4(next(it))[0])
    names = next(it).decode("latin-1")
    type_names = [names[2 * k:2 * k + 2].strip() for k in range(ntypes)]
    E_atom = f8(next(it)).copy()
    normalized = bool(i4(next(it))[0])
    scale = float(f8(next(it))[0])
    shift = float(f8(next(it))[0])
    ts = TrainSet(type_names, E_atom, normalized, scale, shift)
    for _ in range(nstrucs):
        next(it)   # len_trim(filename)
        fname = next(it).decode("latin-1")
        nat, _nt = (int(v) for v in i4(next(it))[:2])
        energy = float(f8(next(it))[0])
        types, coords, forces, sf = [], [], [], []
        for _a in range(nat):
            types.append(int(i4(next(it))[0]))
            coords.append(f8(next(it)).copy())
            forces.append(f8(next(it)).copy())
            nsf = int(i4(next(it))[0])
            v = f8(next(it)).copy()
            if v.size != nsf:
                raise ValueError("%s: descriptor length mismatch" % path)
            sf.append(v)
        ts.add(fname, energy, types, coords, forces, sf)
    next(it)   # nAtomsTot
    ts.E_av, ts.E_min, ts.E_max = (float(v) for v in f8(next(it))[:3])
    has_setups = bool(i4(next(it))[0])
    if has_setups:
        rest = list(it)
        per = len(rest) // ntypes
        ts.setup_records = []
        for k in range(ntypes):
            chunk = rest[k * per:(k + 1) * per]
            ts.setup_records.append(chunk[1:])    # drop the itype record
    return ts


def write_trainset(path, ts):
    out = [_rec(struct.pack("<i", len(ts.type_names))), _rec(struct.pack("<i", len(ts.structures))),
           _rec("".join("%-2s" % t for t in ts.type_names).encode("latin-1")),
           _rec(np.asarray(ts.E_atom, dtype="<f8").tobytes()),
           _rec(struct.pack("<i", 1 if ts.normalized else 0)),
           _rec(struct.pack("<d", ts.scale)), _rec(struct.pack("<d", ts.shift))]
    for s in ts.structures:
        name = s["file"].encode("latin-1")
        out += [_rec(struct.pack("<i", len(name))), _rec(name),
                _rec(struct.pack("<ii", len(s["types"]), len(ts.type_names))),
                _rec(struct.pack("<d", s["energy"]))]
        for a in range(len(s["types"])):
            out += [_rec(struct.pack("<i", int(s["types"][a]))),
                    _rec(np.asarray(s["coords"][a], dtype="<f8").tobytes()),
                    _rec(np.asarray(s["forces"][a], dtype="<f8").tobytes()),
                    _rec(struct.pack("<i", len(s["sfval"][a]))),
                    _rec(np.asarray(s["sfval"][a], dtype="<f8").tobytes())]
    out += [_rec(struct.pack("<i", ts.natoms_total)),
            _rec(struct.pack("<ddd", ts.E_av, ts.E_min, ts.E_max))]
    if ts.setup_records:
        out.append(_rec(struct.pack("<i", 1)))
        for k, recs in enumerate(ts.setup_records, start=1):
            out.append(_rec(struct.pack("<i", k)))
            out += [_rec(r) for r in recs]
    else:
        out.append(_rec(struct.pack("<i", 0)))
    with open(path, "wb") as fh:
        fh.write(b"".join(out))


def normalize(ts, stats, maxenergy=None, scale=None, shift=None):
    """ts_normalize: a new, normalised TrainSet.  ``stats`` maps species
    index (1-based) to (shift, 1/s) arrays of the setups' normalisation
    (stp_normalize); high-energy structures beyond ``maxenergy`` per atom
    are dropped as the reference drops them.  ``scale``/``shift`` override
    the energy normalisation (e.g. to match existing potentials)."""
    E_max = ts.E_max if maxenergy is None else min(ts.E_max, maxenergy)
    if scale is None:
        scale = 2.0 / (E_max - ts.E_min)
    if shift is None:
        shift = 0.5 * (E_max + ts.E_min)
    out = TrainSet(ts.type_names, ts.E_atom, True, scale, shift)
    for s in ts.structures:
        n = len(s["types"])
        e = scale * (s["energy"] - n * shift)
        if maxenergy is not None and e / n > 1.001:
            continue
        sf = [(v - stats[t][0][:len(v)]) * stats[t][1][:len(v)]
              for t, v in zip(s["types"], s["sfval"])]
        out.add(s["file"], e, s["types"], s["coords"], scale * s["forces"], sf)
    out.E_av, out.E_min, out.E_max = ts.E_av, ts.E_min, ts.E_max
    out.setup_records = ts.setup_records
    return out
