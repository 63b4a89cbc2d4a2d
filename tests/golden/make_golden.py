"""Builds tests/golden/chbrclf.npz from the reference repository's own test data.

Sources (read-only, in the reference checkout):
  tests/chbrclf.hpp        CHBrClF molecule: nuclei, AO basis, MO coefficients, electrons
  tests/mo_reference.txt   every mo_vgl[136][5][224] value, compared at 1e-14 absolute
                           by tests/test_qmckl_mo.cpp:382-405
  tests/test_qmckl_ao.cpp  known answers ao_value[26][219..222] (lines 440-448)
  tests/test_qmckl_mo.cpp  known answers ao_vgl[26][0..4][219] (lines 250-259)

The arrays are stored unchanged (same dtypes, same C index order); the known answers
are parsed out of the test sources so that nothing is typed in by hand.

    python tests/golden/make_golden.py [/path/to/reference]
"""
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _numbers(text):
    return [float(t) for t in re.findall(r"[-+]?\d+\.?\d*(?:[eE][-+]?\d+)?", text)]


def parse_header(path):
    src = open(path).read()
    defines = {}
    for m in re.finditer(r"#define\s+(chbrclf_\w+)\s+\(?\s*(?:\(int64_t\))?\s*(\d+)\s*\)?", src):
        defines[m.group(1)] = int(m.group(2))
    arrays = {}
    pat = re.compile(r"(double|int64_t|int32_t)\s+(chbrclf_\w+)((?:\[[^\]]*\])+)\s*=\s*\{", re.S)
    for m in pat.finditer(src):
        ctype, name = m.group(1), m.group(2)
        # find the matching closing brace
        i, depth = m.end() - 1, 0
        while True:
            c = src[i]
            if c == "{":
                depth += 1
            elif c == "}":
                depth -= 1
                if depth == 0:
                    break
            i += 1
        body = src[m.end():i]
        body = re.sub(r"//[^\n]*", "", body)
        vals = _numbers(body)
        dt = {"double": np.float64, "int64_t": np.int64, "int32_t": np.int32}[ctype]
        arrays[name] = np.array(vals, dtype=dt)
    return defines, arrays


def parse_kats(ao_test, mo_test):
    ao_src = open(ao_test).read()
    mo_src = open(mo_test).read()
    ao_value = []
    for m in re.finditer(r"fabs\(ao_value\[AO_VALUE_ID\((\d+),\s*(\d+)\)\]\s*-\s*\(([-+0-9.eE]+)\)\)\s*>\s*\n?\s*([0-9.eE+-]+)", ao_src):
        ao_value.append((int(m.group(1)), int(m.group(2)), float(m.group(3)), float(m.group(4))))
    ao_vgl = []
    for m in re.finditer(r"fabs\(ao_vgl\[AO_VGL_ID\((\d+),\s*(\d+),\s*(\d+)\)\]\s*-\s*\(([-+0-9.eE]+)\)\)\s*>\s*([0-9.eE+-]+)", mo_src):
        ao_vgl.append((int(m.group(1)), int(m.group(2)), int(m.group(3)), float(m.group(4)), float(m.group(5))))
    return ao_value, ao_vgl


def main(ref):
    d, a = parse_header(os.path.join(ref, "tests", "chbrclf.hpp"))
    nucl, shell, prim, ao = (d["chbrclf_nucl_num"], d["chbrclf_shell_num"], d["chbrclf_prim_num"],
                             d["chbrclf_ao_num"])
    mo, walk, elec = d["chbrclf_mo_num"], d["chbrclf_walk_num"], d["chbrclf_elec_num"]
    mo_ref = np.loadtxt(os.path.join(ref, "tests", "mo_reference.txt"))
    ao_value_kat, ao_vgl_kat = parse_kats(os.path.join(ref, "tests", "test_qmckl_ao.cpp"),
                                          os.path.join(ref, "tests", "test_qmckl_mo.cpp"))
    assert len(ao_value_kat) == 4 and len(ao_vgl_kat) == 5, (ao_value_kat, ao_vgl_kat)
    out = dict(
        nucl_num=np.int64(nucl), shell_num=np.int64(shell), prim_num=np.int64(prim), ao_num=np.int64(ao),
        mo_num=np.int64(mo), walk_num=np.int64(walk), elec_num=np.int64(elec),
        elec_up_num=np.int64(d["chbrclf_elec_up_num"]), elec_dn_num=np.int64(d["chbrclf_elec_dn_num"]),
        charge=a["chbrclf_charge"],
        nucl_coord=a["chbrclf_nucl_coord"].reshape(3, nucl),
        nucleus_index=a["chbrclf_basis_nucleus_index"],
        nucleus_shell_num=a["chbrclf_basis_nucleus_shell_num"],
        shell_ang_mom=a["chbrclf_basis_shell_ang_mom"],
        shell_prim_num=a["chbrclf_basis_shell_prim_num"],
        shell_prim_index=a["chbrclf_basis_shell_prim_index"],
        shell_factor=a["chbrclf_basis_shell_factor"],
        ao_factor=a["chbrclf_basis_ao_factor"],
        exponent=a["chbrclf_basis_exponent"],
        coefficient=a["chbrclf_basis_coefficient"],
        prim_factor=a["chbrclf_basis_prim_factor"],
        mo_coef=a["chbrclf_mo_coef"].reshape(mo, ao),
        elec_coord=a["chbrclf_elec_coord"].reshape(walk, elec, 3),
        mo_vgl_ref=mo_ref.reshape(walk * elec, 5, mo),
        kat_ao_value=np.array([k[:3] for k in ao_value_kat], dtype=np.float64),
        kat_ao_value_tol=np.float64(ao_value_kat[0][3]),
        kat_ao_vgl=np.array([k[:4] for k in ao_vgl_kat], dtype=np.float64),
        kat_ao_vgl_tol=np.float64(ao_vgl_kat[0][4]),
    )
    for k, n in [("shell_ang_mom", shell), ("shell_prim_num", shell), ("exponent", prim), ("ao_factor", ao)]:
        assert out[k].size == n, (k, out[k].size, n)
    np.savez_compressed(os.path.join(HERE, "chbrclf.npz"), **out)
    print("wrote", os.path.join(HERE, "chbrclf.npz"))


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    else:
        sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
        from oracle import oracle

        ref = oracle.reference_dir()
        if ref is None:
            sys.exit("reference checkout not found: pass its path or set QMCKL_REFERENCE_DIR")
        main(ref)
