"""Molecular systems for the basis-evaluation path: a plain container in the reference's
array layouts, and seeded synthetic generators for the benchmark workloads.

Layouts (the reference's, C index order):
  nucl_coord [3][nucl_num]  (set with transp 'T')
  coord      [point_num][3] (set with transp 'N')
  mo_coef    [mo_num][ao_num]
Shells are contiguous per nucleus and primitives contiguous per shell, as in the
reference's CHBrClF fixture (tests/chbrclf.hpp:14-40 of the reference).

Synthetic workloads (no public benchmark exists for this path; these stand in with the
shapes and value distributions the benchmark configurations name):
  small   6 nuclei (Z in 1..8) in a 6-bohr cube, 60 s/p/d shells (~120 AOs), 1-5 primitives,
          exponents log-uniform [0.05, 50], coefficients U(0.1, 1), 40 MOs ~ N(0, 1/sqrt(ao)),
          50 points ~ N(nucleus, 1.5^2)
  medium  40 nuclei (Z in 1..10) in a 15-bohr cube, 600 s/p/d/f shells (~1200 AOs), 1-6
          primitives, exponents log-uniform [0.03, 80], 300 MOs, 256 walkers x 160
          electrons = 40960 points ~ N(nucleus, 2^2)
  batched 64 molecules, 5-60 nuclei, 100-1500 AOs, 20-400 MOs, small-config generators,
          32 walkers x 2*nuclei electrons each
  adjoint 8 nuclei, ~200 AOs, 64 MOs, 2048 points
  contracted  generally contracted basis (the form of ANO and correlation-consistent sets):
          per nucleus one set of primitive exponents per angular momentum (10 s, 8 p, 5 d,
          3 f, log-uniform [0.05, 50]) shared by all shells of that angular momentum
          (5 s, 4 p, 3 d, 2 f shells, coefficients U(-1, 1)); 20 nuclei in a 12-bohr cube
          (1100 AOs, 2060 primitives, 26 distinct exponents per nucleus), 300 MOs, points
          ~ N(nucleus, 1.5^2)
"""
from dataclasses import dataclass, field

import numpy as np


def ncart(l):
    """Number of Cartesian functions of angular momentum l."""
    return (l + 1) * (l + 2) // 2


@dataclass
class System:
    nucl_num: int
    charge: np.ndarray
    nucl_coord: np.ndarray  # [3][N]
    shell_num: int
    prim_num: int
    ao_num: int
    nucleus_index: np.ndarray  # int64 [N]
    nucleus_shell_num: np.ndarray  # int64 [N]
    shell_ang_mom: np.ndarray  # int32 [S]
    shell_prim_num: np.ndarray  # int64 [S]
    shell_prim_index: np.ndarray  # int64 [S]
    shell_factor: np.ndarray  # [S]
    exponent: np.ndarray  # [K]
    coefficient: np.ndarray  # [K]
    prim_factor: np.ndarray  # [K]
    ao_factor: np.ndarray  # [A]
    mo_num: int
    mo_coef: np.ndarray  # [M][A]
    coord: np.ndarray  # [P][3]
    name: str = "system"
    meta: dict = field(default_factory=dict)

    @property
    def point_num(self):
        return int(self.coord.shape[0])

    def with_points(self, coord):
        d = dict(self.__dict__)
        d["coord"] = np.ascontiguousarray(coord, dtype=np.float64)
        return System(**d)

    @staticmethod
    def from_npz(path, points="all"):
        """Loads the CHBrClF fixture written by tests/golden/make_golden.py."""
        z = np.load(path)
        coord = z["elec_coord"].reshape(-1, 3)
        if points == "walker0":
            coord = z["elec_coord"][0]
        return System(
            nucl_num=int(z["nucl_num"]), charge=z["charge"].copy(), nucl_coord=np.ascontiguousarray(z["nucl_coord"]),
            shell_num=int(z["shell_num"]), prim_num=int(z["prim_num"]), ao_num=int(z["ao_num"]),
            nucleus_index=z["nucleus_index"].astype(np.int64), nucleus_shell_num=z["nucleus_shell_num"].astype(np.int64),
            shell_ang_mom=z["shell_ang_mom"].astype(np.int32), shell_prim_num=z["shell_prim_num"].astype(np.int64),
            shell_prim_index=z["shell_prim_index"].astype(np.int64), shell_factor=z["shell_factor"].copy(),
            exponent=z["exponent"].copy(), coefficient=z["coefficient"].copy(), prim_factor=z["prim_factor"].copy(),
            ao_factor=z["ao_factor"].copy(), mo_num=int(z["mo_num"]), mo_coef=np.ascontiguousarray(z["mo_coef"]),
            coord=np.ascontiguousarray(coord), name="chbrclf")


def make_system(seed, nucl_num, charge_max, cube, shell_num, l_weights, prim_max, expo_range, mo_num,
                point_num, sigma, coef_range=(0.1, 1.0), name="synthetic", rng=None):
    """Seeded synthetic molecule + points. l_weights[l] is the probability of angular
    momentum l for each shell; every nucleus gets at least one shell."""
    rng = np.random.default_rng(seed) if rng is None else rng
    N = int(nucl_num)
    charge = rng.integers(1, charge_max + 1, size=N).astype(np.float64)
    nucl_coord = rng.uniform(0.0, cube, size=(3, N))
    S = int(shell_num)
    owner = np.concatenate([np.arange(N), rng.integers(0, N, size=S - N)])
    owner.sort()
    l_w = np.asarray(l_weights, dtype=np.float64)
    l_w = l_w / l_w.sum()
    ang = rng.choice(len(l_w), size=S, p=l_w).astype(np.int32)
    # s shells first on each nucleus, then p, d, ... (ordered like real basis sets)
    order = np.lexsort((ang, owner))
    owner, ang = owner[order], ang[order]
    nprim = rng.integers(1, prim_max + 1, size=S).astype(np.int64)
    K = int(nprim.sum())
    shell_prim_index = np.concatenate([[0], np.cumsum(nprim)[:-1]]).astype(np.int64)
    nucleus_shell_num = np.bincount(owner, minlength=N).astype(np.int64)
    nucleus_index = np.concatenate([[0], np.cumsum(nucleus_shell_num)[:-1]]).astype(np.int64)
    lo, hi = np.log(expo_range[0]), np.log(expo_range[1])
    exponent = np.exp(rng.uniform(lo, hi, size=K))
    coefficient = rng.uniform(coef_range[0], coef_range[1], size=K)
    A = int(sum(ncart(int(l)) for l in ang))
    M = min(int(mo_num), A)
    mo_coef = rng.normal(0.0, 1.0 / np.sqrt(A), size=(M, A))
    P = int(point_num)
    centers = rng.integers(0, N, size=P)
    coord = nucl_coord[:, centers].T + rng.normal(0.0, sigma, size=(P, 3))
    return System(
        nucl_num=N, charge=charge, nucl_coord=np.ascontiguousarray(nucl_coord), shell_num=S, prim_num=K, ao_num=A,
        nucleus_index=nucleus_index, nucleus_shell_num=nucleus_shell_num, shell_ang_mom=ang,
        shell_prim_num=nprim, shell_prim_index=shell_prim_index, shell_factor=np.ones(S), exponent=exponent,
        coefficient=coefficient, prim_factor=np.ones(K), ao_factor=np.ones(A), mo_num=M,
        mo_coef=np.ascontiguousarray(mo_coef), coord=np.ascontiguousarray(coord), name=name,
        meta=dict(seed=seed, cube=cube, sigma=sigma, expo_range=tuple(expo_range), prim_max=prim_max,
                  l_weights=tuple(float(x) for x in l_w)))


# s/p/d weights giving ~2.05 AOs per shell (60 shells -> ~120 AOs)
SPD_WEIGHTS = (0.55, 0.40, 0.05)
# s/p/d/f weights giving ~2.08 AOs per shell (600 shells -> ~1200 AOs)
SPDF_WEIGHTS = (0.62, 0.30, 0.06, 0.02)


def with_empty_nucleus(s, at, xyz=(0.7, -1.1, 0.3), charge=1.0):
    """s with one more centre, inserted at position `at`, that owns no shell (a bare charge): its
    nucleus_index entry is 0 and its shell count 0. Its AO and MO values are those of s."""
    d = dict(s.__dict__)
    ins = lambda a, v: np.insert(np.asarray(a), at, v)
    d["nucl_num"] = s.nucl_num + 1
    d["charge"] = ins(s.charge, charge)
    d["nucl_coord"] = np.ascontiguousarray(np.insert(s.nucl_coord, at, list(xyz), axis=1))
    d["nucleus_index"] = ins(s.nucleus_index, 0).astype(np.int64)
    d["nucleus_shell_num"] = ins(s.nucleus_shell_num, 0).astype(np.int64)
    d["name"] = "%s+empty@%d" % (s.name, at)
    return System(**d)


def config_small(seed=0, point_num=50):
    return make_system(seed, 6, 8, 6.0, 60, SPD_WEIGHTS, 5, (0.05, 50.0), 40, point_num, 1.5, name="small")


def config_medium(seed=0, walkers=256, electrons=160):
    return make_system(seed, 40, 10, 15.0, 600, SPDF_WEIGHTS, 6, (0.03, 80.0), 300, walkers * electrons, 2.0,
                       name="medium")


def config_adjoint(seed=0):
    cube = 6.0 * (8 / 6.0) ** (1.0 / 3.0)
    return make_system(seed, 8, 8, cube, 98, SPD_WEIGHTS, 5, (0.05, 50.0), 64, 2048, 1.5, name="adjoint")


def config_batched(seed=0, molecules=64, walkers=32):
    """64 molecules of uneven size; cube edge grows as N^(1/3) to keep the small config's
    nuclear density. Returns a list of Systems."""
    rng = np.random.default_rng(seed)
    out = []
    for m in range(molecules):
        N = int(rng.integers(5, 61))
        A_target = int(rng.integers(100, 1501))
        S = max(N, int(round(A_target / 2.05)))
        M = int(rng.integers(20, 401))
        cube = 6.0 * (N / 6.0) ** (1.0 / 3.0)
        P = walkers * 2 * N
        out.append(make_system(None, N, 8, cube, S, SPD_WEIGHTS, 5, (0.05, 50.0), M, P, 1.5,
                               name="batched[%d]" % m, rng=rng))
    return out


def config_contracted(seed=0, point_num=40960, nucl_num=20, mo_num=300):
    """Generally contracted synthetic basis: shells of one angular momentum on a nucleus share
    that nucleus' primitive exponents and differ in their coefficients."""
    rng = np.random.default_rng(seed)
    N = int(nucl_num)
    charge = rng.integers(1, 11, size=N).astype(np.float64)
    nucl_coord = rng.uniform(0.0, 12.0, size=(3, N))
    layout = ((0, 5, 10), (1, 4, 8), (2, 3, 5), (3, 2, 3))  # (l, shells, primitives per shell)
    ang, nprim, expo, coef, nsh = [], [], [], [], []
    for n in range(N):
        cnt = 0
        for l, shells, k in layout:
            ex = np.sort(np.exp(rng.uniform(np.log(0.05), np.log(50.0), size=k)))[::-1]
            for _ in range(shells):
                ang.append(l)
                nprim.append(k)
                expo.append(ex)
                coef.append(rng.uniform(-1.0, 1.0, size=k))
                cnt += 1
        nsh.append(cnt)
    ang = np.asarray(ang, np.int32)
    nprim = np.asarray(nprim, np.int64)
    S, K = len(ang), int(nprim.sum())
    nucleus_shell_num = np.asarray(nsh, np.int64)
    nucleus_index = np.concatenate([[0], np.cumsum(nucleus_shell_num)[:-1]]).astype(np.int64)
    shell_prim_index = np.concatenate([[0], np.cumsum(nprim)[:-1]]).astype(np.int64)
    A = int(sum(ncart(int(l)) for l in ang))
    M = min(int(mo_num), A)
    mo_coef = rng.normal(0.0, 1.0 / np.sqrt(A), size=(M, A))
    centers = rng.integers(0, N, size=int(point_num))
    coord = nucl_coord[:, centers].T + rng.normal(0.0, 1.5, size=(int(point_num), 3))
    return System(
        nucl_num=N, charge=charge, nucl_coord=np.ascontiguousarray(nucl_coord), shell_num=S, prim_num=K, ao_num=A,
        nucleus_index=nucleus_index, nucleus_shell_num=nucleus_shell_num, shell_ang_mom=ang, shell_prim_num=nprim,
        shell_prim_index=shell_prim_index, shell_factor=np.ones(S), exponent=np.concatenate(expo),
        coefficient=np.concatenate(coef), prim_factor=np.ones(K), ao_factor=np.ones(A), mo_num=M,
        mo_coef=np.ascontiguousarray(mo_coef), coord=np.ascontiguousarray(coord), name="contracted",
        meta=dict(seed=seed, layout=layout))
