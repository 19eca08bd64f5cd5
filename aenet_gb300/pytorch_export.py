"""generate.x's PyTorch export: descriptor Jacobians for force training.

File layout (`<training-set file>.forces`, Fortran unformatted sequential
records, little endian), as pytorchoutput.f90 writes it:

  header      nStrucs                                   (pyo_write_header_info)
  structure   len_trim(filename) | filename | nAtoms, nTypes |
              forces-selected flag (0/1)                (pyo_write_structure_info)
  per atom of a selected structure:
              itype | nsf, nnb | nblist(1:nnb) |
              sfderiv_i(1:nsf, 1:3) | sfderiv_j(1:nnb, 1:nsf, 1:3)
              (column-major, pyo_write_atom_sf_info, pytorchoutput.f90:104-138)
  footer      largest nnb written                       (pyo_write_final)

The derivatives are those of the raw (unnormalised) descriptors, as
stp_eval returns them to generate.x; nblist holds 1-based atom indices of
the structure (periodic images repeat an index).  The neighbours come in
the GPU search's order, not lclist's: consumers pair nblist with the
sfderiv_j rows, so the order carries no meaning.  Structures are selected
as pyo_select_force_structures does (the first round(n * fraction) flags
set, then shuffled) with numpy's generator instead of the Fortran one.
"""
import struct

import numpy as np

__all__ = ["select_structures", "write_forces_file", "read_forces_file"]


def _rec(payload):
    return struct.pack("<i", len(payload)) + payload + struct.pack("<i", len(payload))


def select_structures(nstrucs, fraction, seed=0):
    """0/1 flags: round(nstrucs * fraction) ones, shuffled."""
    flags = np.zeros(nstrucs, dtype=np.int32)
    flags[:int(np.rint(nstrucs * fraction))] = 1
    return np.random.default_rng(seed).permutation(flags)


def write_forces_file(path, structures):
    """``structures``: dicts with name, natoms, ntypes, selected and, when
    selected, atoms = [(itype, nblist (1-based), dG_i (nsf, 3),
    dG_j (nnb, nsf, 3)), ...].  Returns the largest nnb written."""
    out = [_rec(struct.pack("<i", len(structures)))]
    max_nnb = 0
    for s in structures:
        name = s["name"].encode("latin-1")
        out += [_rec(struct.pack("<i", len(name))), _rec(name),
                _rec(struct.pack("<ii", s["natoms"], s["ntypes"])),
                _rec(struct.pack("<i", 1 if s["selected"] else 0))]
        if not s["selected"]:
            continue
        for itype, nbl, dGi, dGj in s["atoms"]:
            nsf = dGi.shape[0]
            nnb = len(nbl)
            max_nnb = max(max_nnb, nnb)
            out += [_rec(struct.pack("<i", int(itype))), _rec(struct.pack("<ii", nsf, nnb)),
                    _rec(np.asarray(nbl, dtype="<i4").tobytes()),
                    _rec(np.asarray(dGi, dtype="<f8").tobytes(order="F")),
                    _rec(np.asarray(dGj, dtype="<f8").reshape(nnb, nsf, 3).tobytes(order="F"))]
    out.append(_rec(struct.pack("<i", max_nnb)))
    with open(path, "wb") as fh:
        fh.write(b"".join(out))
    return max_nnb


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


def read_forces_file(path):
    """Inverse of :func:`write_forces_file`: (structures, max_nnb)."""
    it = iter(_records(open(path, "rb").read()))
    i4 = lambda r: np.frombuffer(r, "<i4")
    nstrucs = int(i4(next(it))[0])
    structures = []
    for _ in range(nstrucs):
        next(it)
        name = next(it).decode("latin-1")
        natoms, ntypes = (int(v) for v in i4(next(it))[:2])
        selected = bool(i4(next(it))[0])
        atoms = []
        if selected:
            for _a in range(natoms):
                itype = int(i4(next(it))[0])
                nsf, nnb = (int(v) for v in i4(next(it))[:2])
                nbl = i4(next(it)).copy()
                dGi = np.frombuffer(next(it), "<f8").reshape((nsf, 3), order="F").copy()
                dGj = np.frombuffer(next(it), "<f8").reshape((nnb, nsf, 3), order="F").copy()
                atoms.append((itype, nbl, dGi, dGj))
        structures.append({"name": name, "natoms": natoms, "ntypes": ntypes,
                           "selected": selected, "atoms": atoms})
    max_nnb = int(i4(next(it))[0])
    return structures, max_nnb
