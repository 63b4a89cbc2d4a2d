"""The oracle's FP64 reference gradient of L = sum(W * mo_vgl) (adjoint form) against central
finite differences of the oracle's forward path (h = 1e-5), whose parity with the reference is
pinned by the golden tests: dL/dC, dL/dexponent and dL/dcoord within 1e-7 (normwise, relative to
the largest gradient entry). CPU only."""
import numpy as np
import pytest

from oracle import oracle
from qmckl_sycl_gb300 import config_adjoint, config_small

H = 1e-5
FD_RTOL = 1e-7


def loss_per_point(s, w):
    mo = oracle.forward(s, want=("mo_vgl",))["mo_vgl"]
    return (w * mo).sum(axis=(1, 2))


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def replace(s, **kw):
    return s.__class__(**{**s.__dict__, **kw})


@pytest.fixture(scope="module")
def adjoint_case():
    s = config_adjoint(0)
    w = np.random.default_rng(5).normal(size=(s.point_num, 5, s.mo_num))
    return s, w


def test_coord_gradient_matches_central_differences(adjoint_case):
    s, w = adjoint_case
    g = oracle.vjp_mo_vgl(s, w, want=("coord",))["coord"]
    fd = np.zeros_like(g)
    for j in range(3):  # each point's loss depends on its own coordinates only
        e = np.zeros(3)
        e[j] = H
        lp = loss_per_point(s.with_points(s.coord + e), w)
        lm = loss_per_point(s.with_points(s.coord - e), w)
        fd[:, j] = (lp - lm) / (2 * H)
    assert rel(g, fd) <= FD_RTOL


def test_exponent_gradient_matches_central_differences(adjoint_case):
    s, w = adjoint_case
    idx = np.arange(0, s.point_num, 16)  # 128 points keep 2 x 307 forward passes quick
    sub = s.with_points(s.coord[idx])
    wsub = np.ascontiguousarray(w[idx])
    g = oracle.vjp_mo_vgl(sub, wsub, want=("expo",))["expo"]
    fd = np.zeros_like(g)
    for k in range(s.prim_num):
        ep = s.exponent.copy()
        ep[k] += H
        em = s.exponent.copy()
        em[k] -= H
        fd[k] = (loss_per_point(replace(sub, exponent=ep), wsub).sum() -
                 loss_per_point(replace(sub, exponent=em), wsub).sum()) / (2 * H)
    assert rel(g, fd) <= FD_RTOL


def test_coefficient_and_directional_gradients(adjoint_case):
    s, w = adjoint_case
    g = oracle.vjp_mo_vgl(s, w)
    rng = np.random.default_rng(9)
    # L is linear in C: dL/dC = sum_p w_p^T ao_p exactly, check along random directions
    for _ in range(2):
        d = rng.normal(size=g["coef"].shape)
        lp = loss_per_point(replace(s, mo_coef=s.mo_coef + H * d), w).sum()
        lm = loss_per_point(replace(s, mo_coef=s.mo_coef - H * d), w).sum()
        assert abs((lp - lm) / (2 * H) - (g["coef"] * d).sum()) <= FD_RTOL * np.abs(g["coef"]).sum()
    # all exponents at once along a random direction, full point set
    d = rng.normal(size=s.prim_num)
    lp = loss_per_point(replace(s, exponent=s.exponent + H * d), w).sum()
    lm = loss_per_point(replace(s, exponent=s.exponent - H * d), w).sum()
    assert abs((lp - lm) / (2 * H) - (g["expo"] * d).sum()) <= FD_RTOL * np.abs(g["expo"] * d).sum()


def test_d_shells_and_zero_value_mask():
    # the small configuration has d shells; a point on a nucleus makes x = y = z = 0 there,
    # so p and d components vanish exactly and the MO kernel's zero-value skip is exercised
    s = config_small(2, point_num=24)
    coord = s.coord.copy()
    coord[0] = s.nucl_coord[:, 0]
    s = s.with_points(coord)
    w = np.random.default_rng(3).normal(size=(s.point_num, 5, s.mo_num))
    g = oracle.vjp_mo_vgl(s, w, want=("coord", "expo"))
    fd = np.zeros_like(g["coord"])
    for j in range(3):
        e = np.zeros(3)
        e[j] = H
        fd[:, j] = (loss_per_point(s.with_points(s.coord + e), w) -
                    loss_per_point(s.with_points(s.coord - e), w)) / (2 * H)
    # point 0 sits where the mask switches terms on and off: compare the others
    assert rel(g["coord"][1:], fd[1:]) <= FD_RTOL
    fde = np.zeros(s.prim_num)
    for k in range(s.prim_num):
        ep = s.exponent.copy()
        ep[k] += H
        em = s.exponent.copy()
        em[k] -= H
        fde[k] = (loss_per_point(replace(s, exponent=ep), w).sum() -
                  loss_per_point(replace(s, exponent=em), w).sum()) / (2 * H)
    assert rel(g["expo"], fde) <= FD_RTOL
