"""Test infrastructure for the TREXIO reader: builds the libtrexio test double (trexio_double.c)
and writes files in its format, including a system's data in TREXIO's layout (per-shell nucleus
index, per-primitive shell index, nucleus coordinates [nucleus][3], MO coefficients [mo][ao])."""
import os
import struct
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SOURCE = os.path.join(HERE, "trexio_double.c")
_KIND = {np.dtype(np.int64): 1, np.dtype(np.float64): 2, np.dtype(np.int32): 3}


def build(outdir):
    """Compiles the double into outdir/libtrexio.so and returns its path."""
    so = os.path.join(outdir, "libtrexio.so")
    subprocess.run(["gcc", "-O1", "-std=c99", "-Wall", "-Werror", "-shared", "-fPIC", "-o", so, SOURCE], check=True)
    return so


def write(path, records, back_end="T"):
    """Writes {name: value} (int64/float64/int32 arrays or scalars, or a str) to path; back_end 'T'
    makes the double open the file with the text back end, 'H' with HDF5."""
    with open(path, "wb") as f:
        f.write(b"TRXDBL1" + back_end.encode())
        for name, value in records.items():
            if isinstance(value, str):
                kind, payload, count = 4, value.encode(), len(value.encode())
            else:
                a = np.ascontiguousarray(value)
                kind, payload, count = _KIND[a.dtype], a.tobytes(), a.size
            assert len(name) < 48
            f.write(name.encode().ljust(48, b"\0"))
            f.write(struct.pack("<iiq", kind, 0, count))
            f.write(payload)


def owner_of_members(first, count, member_num):
    """The inverse of (first, count) per owner: the owner of each member, -1 where none."""
    owner = np.full(member_num, -1, dtype=np.int64)
    for k, (lo, n) in enumerate(zip(first, count)):
        owner[lo:lo + n] = k
    return owner


def records_of(s, up_num, dn_num, mo=True):
    """A System's data as the TREXIO groups electron, nucleus, basis, ao and mo hold it."""
    r = {
        "electron_up_num": np.int64(up_num),
        "electron_dn_num": np.int64(dn_num),
        "nucleus_num": np.int64(s.nucl_num),
        "nucleus_charge": np.asarray(s.charge, np.float64),
        "nucleus_coord": np.ascontiguousarray(np.asarray(s.nucl_coord, np.float64).T),
        "basis_type": "Gaussian",
        "basis_shell_num": np.int64(s.shell_num),
        "basis_prim_num": np.int64(s.prim_num),
        "basis_nucleus_index": owner_of_members(s.nucleus_index, s.nucleus_shell_num, s.shell_num),
        "basis_shell_ang_mom": np.asarray(s.shell_ang_mom, np.int32),
        "basis_shell_factor": np.asarray(s.shell_factor, np.float64),
        "basis_shell_index": owner_of_members(s.shell_prim_index, s.shell_prim_num, s.prim_num),
        "basis_exponent": np.asarray(s.exponent, np.float64),
        "basis_coefficient": np.asarray(s.coefficient, np.float64),
        "basis_prim_factor": np.asarray(s.prim_factor, np.float64),
        "ao_num": np.int64(s.ao_num),
        "ao_normalization": np.asarray(s.ao_factor, np.float64),
    }
    if mo:
        r["mo_num"] = np.int64(s.mo_num)
        r["mo_coefficient"] = np.ascontiguousarray(np.asarray(s.mo_coef, np.float64))
    return r
