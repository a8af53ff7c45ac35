"""Readers of the snapshot files of Output_plt_file (mpm_ini.cpp:832-980): the
particle Tecplot binary (#!TDV112) and the ASCII cell table."""
import struct

import numpy as np


def read_particle_plt(path):
    """Returns (header dict, {name: array}) of a particle file."""
    b = open(path, "rb").read()
    o = 0

    def take(fmt):
        nonlocal o
        v = struct.unpack_from("<" + fmt, b, o)
        o += struct.calcsize("<" + fmt)
        return v if len(v) > 1 else v[0]

    def name():
        s = []
        while True:
            c = take("i")
            if c == 0:
                return "".join(s)
            s.append(chr(c))

    assert b[:8] == b"#!TDV112"
    o = 8
    hdr = {"version": take("3i"), "nvar": take("i")}
    hdr["names"] = [name() for _ in range(hdr["nvar"])]
    assert take("f") == 299.0
    hdr["zone"] = name()
    hdr["parent_strand"] = take("2i")
    hdr["time"] = take("d")
    hdr["zone_flags"] = take("5i")
    hdr["imax"], hdr["jmax"], hdr["kmax"] = take("3i")
    hdr["aux"] = take("i")
    assert take("f") == 357.0
    assert take("f") == 299.0
    hdr["types"] = list(take(f"{hdr['nvar']}i"))
    hdr["sharing"] = take("3i")
    hdr["ranges"] = take(f"{2 * hdr['nvar']}d")
    n = hdr["imax"]
    data = {}
    for nm, t in zip(hdr["names"], hdr["types"]):
        dt = np.float64 if t == 2 else np.int32
        a = np.frombuffer(b, dtype=dt, count=n, offset=o)
        o += a.nbytes
        data[nm] = a
    assert o == len(b), (o, len(b))
    hdr["data_offset"] = len(b) - sum(a.nbytes for a in data.values())
    return hdr, data


def read_cell_table(path):
    """Returns (the two header lines, array [ncell, 15])."""
    with open(path) as f:
        h1 = f.readline()
        h2 = f.readline()
        rows = np.loadtxt(f, ndmin=2)
    return (h1, h2), rows
