"""aenet ``.nn`` potential files: writer and reader (host side).

The format is the one ``load_NNPot`` reads (src/potential.f90:111-157): a
Fortran unformatted sequential file, every record framed as
``[int32 n][n bytes][int32 n]`` (little endian), holding

* Network  -- nlayers, nnodes_max, Wsize, nvalues, nnodes(:), f_a(2:),
  iw(:), iv(:), W(:)                       (src/ext/feedforward.f90:291-306)
* Setup    -- description, atomtype, nenv, envtypes, Rc_min, Rc_max,
  sftype, nsf, nsfparam, sf(:), sfparam(4,:), sfenv(2,:), neval,
  sfval_min/max/avg(/cov)                   (src/sfsetup.f90:585-609)
* TrnSet info -- file, normalized, scale, shift, nTypes, typeName(:),
  E_atom(:), nAtomsTot, nStrucs, E_min/E_max/E_av
                                            (src/trainset.f90:432-441)

Strings are fixed width and blank padded (description 1024, type names 2,
sftype 100, file 1024).  Files written by old versions of the reference
have 16 Setup records (no ``sfval_cov``); :func:`read_nn` accepts both and
reports ``legacy``.  The GPU library has its own C++ loader behind
``aenet_load_potential``; this module exists to create and inspect files.
"""
import struct

import numpy as np

__all__ = ["make_network", "chebyshev_setup", "behler_setup", "write_nn",
           "read_nn", "network_layout"]


def network_layout(arch):
    """Index bookkeeping of new_Network (src/ext/feedforward.f90:97-149)."""
    arch = [int(a) for a in arch]
    nl = len(arch)
    iw = [0] * nl
    iv = [0] * nl
    wsize = 0
    for l in range(nl - 1):
        wsize += (arch[l] + 1) * arch[l + 1]
        iw[l + 1] = wsize
    nvalues = 0
    for l in range(nl - 1):
        nvalues += arch[l] + 1
        iv[l + 1] = nvalues
    nvalues += arch[-1]
    return {"nlayers": nl, "nnodes": np.array(arch), "nnodes_max": max(arch),
            "Wsize": wsize, "nvalues": nvalues, "iw": np.array(iw),
            "iv": np.array(iv)}


def make_network(arch, W, activations=None):
    """Network dict; ``activations`` are the f_a codes of layers 2..L
    (default: tanh hidden layers, linear output)."""
    net = network_layout(arch)
    if activations is None:
        activations = [1] * (len(arch) - 2) + [0]
    net["f_a"] = np.array(activations)
    W = np.asarray(W, dtype=np.float64).ravel()
    if W.size != net["Wsize"]:
        raise ValueError("expected %d weights, got %d" % (net["Wsize"], W.size))
    net["W"] = W
    return net


def chebyshev_setup(atomtype, envtypes, r_Rc, r_order, a_Rc, a_order,
                    Rc_min, description="Chebyshev descriptor"):
    """Setup dict of the Chebyshev basis (read_basis_chebyshev,
    src/sfsetup.f90:1102-1158); statistics are filled in later."""
    nsf = r_order + a_order + 2
    if len(envtypes) > 1:
        nsf *= 2
    sfparam = np.zeros((nsf, 4))
    sfparam[0] = [r_Rc, float(r_order), a_Rc, float(a_order)]
    return {"description": description, "atomtype": atomtype,
            "nenv": len(envtypes), "envtypes": list(envtypes),
            "Rc_min": float(Rc_min), "Rc_max": float(max(r_Rc, a_Rc)),
            "sftype": "Chebyshev", "nsf": nsf, "nsfparam": 4,
            "sf": np.zeros(nsf, dtype=np.int64), "sfparam": sfparam,
            "sfenv": np.zeros((nsf, 2), dtype=np.int64), "neval": 0,
            "sfval_min": np.zeros(nsf), "sfval_max": np.zeros(nsf),
            "sfval_avg": np.zeros(nsf), "sfval_cov": np.zeros(nsf)}


def behler_setup(atomtype, envtypes, functions, Rc_min,
                 description="Behler2011 symmetry functions"):
    """Setup dict of Behler2011 functions (read_symmfunc_Behler2011,
    src/sfsetup.f90:1222-1280).  ``functions`` is a list of dicts such as
    ``{"G": 2, "type2": "O", "Rc": 6.5, "Rs": 0.0, "eta": 0.1}`` or
    ``{"G": 4, "type2": "O", "type3": "Ti", "Rc": 6.5, "lambda": 1,
    "zeta": 2, "eta": 0.01}``, in file order."""
    nsf = len(functions)
    sf = np.zeros(nsf, dtype=np.int64)
    sfparam = np.zeros((nsf, 4))
    sfenv = np.zeros((nsf, 2), dtype=np.int64)
    rc_max = 0.0
    for i, f in enumerate(functions):
        g = int(f["G"])
        sf[i] = g
        sfenv[i, 0] = envtypes.index(f["type2"]) + 1
        if g in (4, 5):
            sfenv[i, 1] = envtypes.index(f["type3"]) + 1
        if g == 1:
            sfparam[i, 0] = f["Rc"]
        elif g == 2:
            sfparam[i, :3] = [f["Rc"], f["Rs"], f["eta"]]
        elif g == 3:
            sfparam[i, :2] = [f["Rc"], f["kappa"]]
        elif g in (4, 5):
            sfparam[i] = [f["Rc"], f["lambda"], f["zeta"], f["eta"]]
        else:
            raise ValueError("unknown symmetry function G%d" % g)
        rc_max = max(rc_max, float(f["Rc"]))
    return {"description": description, "atomtype": atomtype,
            "nenv": len(envtypes), "envtypes": list(envtypes),
            "Rc_min": float(Rc_min), "Rc_max": rc_max, "sftype": "Behler2011",
            "nsf": nsf, "nsfparam": 4, "sf": sf, "sfparam": sfparam,
            "sfenv": sfenv, "neval": 0, "sfval_min": np.zeros(nsf),
            "sfval_max": np.zeros(nsf), "sfval_avg": np.zeros(nsf),
            "sfval_cov": np.zeros(nsf)}


def _rec(payload):
    n = len(payload)
    return struct.pack("<i", n) + payload + struct.pack("<i", n)


def _i4(v):
    return _rec(np.asarray(v, dtype="<i4").tobytes())


def _f8(v):
    return _rec(np.asarray(v, dtype="<f8").tobytes())


def _s(text, width):
    b = text.encode("latin-1")[:width]
    return _rec(b + b" " * (width - len(b)))


def setup_payloads(stp, legacy=False):
    """The Setup records of save_Setup (src/sfsetup.f90:585-609) as raw
    payloads (no record framing), as potential and training-set files
    store them."""
    env = "".join("%-2s" % e for e in stp["envtypes"])
    pay = lambda rec: rec[4:-4]
    out = [_s(stp["description"], 1024), _s(stp["atomtype"], 2),
           _i4([stp["nenv"]]), _rec(env.encode("latin-1")),
           _f8([stp["Rc_min"]]), _f8([stp["Rc_max"]]), _s(stp["sftype"], 100),
           _i4([stp["nsf"]]), _i4([stp["nsfparam"]]), _i4(stp["sf"]),
           _f8(np.asarray(stp["sfparam"]).ravel()),
           _i4(np.asarray(stp["sfenv"]).ravel()), _i4([stp.get("neval", 0)]),
           _f8(stp["sfval_min"]), _f8(stp["sfval_max"]), _f8(stp["sfval_avg"])]
    if not legacy:
        out.append(_f8(stp["sfval_cov"]))
    return [pay(r) for r in out]


def write_nn(path, net, stp, ts, legacy=False):
    """Write a potential file.  ``ts`` needs keys scale, shift, typeName,
    E_atom (others default).  ``legacy=True`` omits ``sfval_cov``."""
    out = []
    out += [_i4([net["nlayers"]]), _i4([net["nnodes_max"]]), _i4([net["Wsize"]]),
            _i4([net["nvalues"]]), _i4(net["nnodes"]), _i4(net["f_a"]),
            _i4(net["iw"]), _i4(net["iv"]), _f8(net["W"])]
    env = "".join("%-2s" % e for e in stp["envtypes"])
    out += [_s(stp["description"], 1024), _s(stp["atomtype"], 2),
            _i4([stp["nenv"]]), _rec(env.encode("latin-1")),
            _f8([stp["Rc_min"]]), _f8([stp["Rc_max"]]), _s(stp["sftype"], 100),
            _i4([stp["nsf"]]), _i4([stp["nsfparam"]]), _i4(stp["sf"]),
            _f8(np.asarray(stp["sfparam"]).ravel()),
            _i4(np.asarray(stp["sfenv"]).ravel()), _i4([stp.get("neval", 0)]),
            _f8(stp["sfval_min"]), _f8(stp["sfval_max"]), _f8(stp["sfval_avg"])]
    if not legacy:
        out.append(_f8(stp["sfval_cov"]))
    names = "".join("%-2s" % t for t in ts["typeName"])
    out += [_s(ts.get("file", "synthetic"), 1024),
            _i4([int(ts.get("normalized", True))]), _f8([ts["scale"]]),
            _f8([ts["shift"]]), _i4([len(ts["typeName"])]),
            _rec(names.encode("latin-1")), _f8(ts["E_atom"]),
            _i4([ts.get("nAtomsTot", 0)]), _i4([ts.get("nStrucs", 0)]),
            _f8([ts.get("E_min", 0.0), ts.get("E_max", 0.0), ts.get("E_av", 0.0)])]
    with open(path, "wb") as fh:
        fh.write(b"".join(out))


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


def read_nn(path):
    """Parse a potential file into (net, stp, ts, legacy)."""
    recs = _records(open(path, "rb").read())
    if len(recs) not in (35, 36):
        raise ValueError("%s: %d records, expected 35 or 36" % (path, len(recs)))
    legacy = len(recs) == 35
    it = iter(recs)
    i4 = lambda: np.frombuffer(next(it), "<i4").astype(np.int64)
    f8 = lambda: np.frombuffer(next(it), "<f8").astype(np.float64)
    s = lambda: next(it).decode("latin-1")
    net = {"nlayers": int(i4()[0]), "nnodes_max": int(i4()[0]),
           "Wsize": int(i4()[0]), "nvalues": int(i4()[0])}
    net["nnodes"], net["f_a"], net["iw"], net["iv"], net["W"] = i4(), i4(), i4(), i4(), f8()
    stp = {"description": s().rstrip(), "atomtype": s().strip(), "nenv": int(i4()[0])}
    env = s()
    stp["envtypes"] = [env[2 * k:2 * k + 2].strip() for k in range(stp["nenv"])]
    stp["Rc_min"], stp["Rc_max"] = float(f8()[0]), float(f8()[0])
    stp["sftype"] = s().strip()
    stp["nsf"], stp["nsfparam"] = int(i4()[0]), int(i4()[0])
    stp["sf"] = i4()
    stp["sfparam"] = f8().reshape(stp["nsf"], stp["nsfparam"])
    stp["sfenv"] = i4().reshape(stp["nsf"], -1)
    stp["neval"] = int(i4()[0])
    stp["sfval_min"], stp["sfval_max"], stp["sfval_avg"] = f8(), f8(), f8()
    stp["sfval_cov"] = None if legacy else f8()
    ts = {"file": s().rstrip(), "normalized": bool(i4()[0]),
          "scale": float(f8()[0]), "shift": float(f8()[0])}
    nt = int(i4()[0])
    names = s()
    ts["typeName"] = [names[2 * k:2 * k + 2].strip() for k in range(nt)]
    ts["E_atom"] = f8()
    ts["nAtomsTot"], ts["nStrucs"] = int(i4()[0]), int(i4()[0])
    ts["E_min"], ts["E_max"], ts["E_av"] = (float(x) for x in f8())
    return net, stp, ts, legacy
