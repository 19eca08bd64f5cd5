"""Reader for aenet ``.nn`` potential files -- oracle side, test infrastructure.

A ``.nn`` file is a Fortran unformatted sequential file (every record is
``[int32 n][n bytes][int32 n]``, little endian) holding, in order:

* the Network   (feedforward.f90:291-306, 9 records),
* the Setup     (sfsetup.f90:585-609, 17 records; legacy files have 16,
                 without ``sfval_cov``),
* the TrnSet info block (trainset.f90:432-441, 10 records).

This parser is independent of the product library's C++ loader so that the
two can be checked against each other.
"""
import struct

import numpy as np


def read_records(path):
    data = open(path, "rb").read()
    recs, i = [], 0
    while i < len(data):
        (n,) = struct.unpack_from("<i", data, i)
        payload = data[i + 4:i + 4 + n]
        (m,) = struct.unpack_from("<i", data, i + 4 + n)
        if m != n:
            raise ValueError("corrupt record marker in %s" % path)
        recs.append(payload)
        i += 8 + n
    return recs


def _i4(b):
    return np.frombuffer(b, dtype="<i4").astype(np.int64)


def _f8(b):
    return np.frombuffer(b, dtype="<f8").astype(np.float64)


def _str(b):
    return b.decode("latin-1")


def parse_nn(path):
    recs = read_records(path)
    if len(recs) not in (35, 36):
        raise ValueError("unexpected record count %d in %s" % (len(recs), path))
    legacy = len(recs) == 35
    r = iter(recs)
    net = {}
    net["nlayers"] = int(_i4(next(r))[0])
    net["nnodes_max"] = int(_i4(next(r))[0])
    net["Wsize"] = int(_i4(next(r))[0])
    net["nvalues"] = int(_i4(next(r))[0])
    net["nnodes"] = _i4(next(r))
    net["f_a"] = _i4(next(r))
    net["iw"] = _i4(next(r))
    net["iv"] = _i4(next(r))
    net["W"] = _f8(next(r))
    stp = {}
    stp["description"] = _str(next(r)).rstrip()
    stp["atomtype"] = _str(next(r)).strip()
    stp["nenv"] = int(_i4(next(r))[0])
    env = _str(next(r))
    stp["envtypes"] = [env[2 * k:2 * k + 2].strip() for k in range(stp["nenv"])]
    stp["Rc_min"] = float(_f8(next(r))[0])
    stp["Rc_max"] = float(_f8(next(r))[0])
    stp["sftype"] = _str(next(r)).strip()
    stp["nsf"] = nsf = int(_i4(next(r))[0])
    stp["nsfparam"] = int(_i4(next(r))[0])
    stp["sf"] = _i4(next(r))
    stp["sfparam"] = _f8(next(r)).reshape(nsf, stp["nsfparam"])
    stp["sfenv"] = _i4(next(r)).reshape(nsf, -1)
    stp["neval"] = int(_i4(next(r))[0])
    stp["sfval_min"] = _f8(next(r))
    stp["sfval_max"] = _f8(next(r))
    stp["sfval_avg"] = _f8(next(r))
    stp["sfval_cov"] = None if legacy else _f8(next(r))
    ts = {}
    ts["file"] = _str(next(r)).rstrip()
    ts["normalized"] = bool(_i4(next(r))[0])
    ts["scale"] = float(_f8(next(r))[0])
    ts["shift"] = float(_f8(next(r))[0])
    ts["nTypes"] = nt = int(_i4(next(r))[0])
    names = _str(next(r))
    ts["typeName"] = [names[2 * k:2 * k + 2].strip() for k in range(nt)]
    ts["E_atom"] = _f8(next(r))
    ts["nAtomsTot"] = int(_i4(next(r))[0])
    ts["nStrucs"] = int(_i4(next(r))[0])
    ts["E_min"], ts["E_max"], ts["E_av"] = (float(x) for x in _f8(next(r)))
    return {"net": net, "stp": stp, "ts": ts, "legacy": legacy}
