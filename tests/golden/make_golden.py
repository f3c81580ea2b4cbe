"""Writes tests/golden/reference_fixtures.json: the known-answer data of So-bogus's own unit tests for the
friction-solve path, restated as plain numbers. Each entry names the reference test it comes from.

The reference cannot be compiled here (it needs Eigen and googletest, both fetched at configure time), so its
tests are read as text: the fixture inputs and the expected values below are the reference's; the derived
arrays (b, W, padded H) follow the steps those tests perform.

Run:  python tests/golden/make_golden.py
"""
import json
import os

import numpy as np


def small_friction_pb():
    """tests/SmallFrictionPb.hpp:18-67 — 2 bodies (4 and 2 dofs), 2 contacts, mu = (0.5, 0.7)."""
    dofs = [4, 2]
    M0 = np.eye(4)
    M1 = np.diag([2.0, 2.0])
    H00 = np.array([3, 5, 7, -1, 2, 4, 5, 4, 1, 6, 9, 1], float).reshape(3, 4)
    H01 = np.array([-3, -6, -6, -5, -5, -8], float).reshape(3, 2)
    H10 = np.array([3, 7, 1, -1, 3, 6, 3, 2, 4, 4, 7, -1], float).reshape(3, 4)
    H2B = np.array([6, 7, 10, 9, 5, 8, 11, 8, 4, 9, 12, 7], float).reshape(3, 4)
    E = np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0]], float)
    H10 = E.T @ (H10 - H2B)  # H.block(2) -= H2B; H.block(2) = E^T H.block(2)
    f = np.array([1, 2, 3, 4, 5, 6], float)
    w = np.array([2, 1, 2, 1, 3, 3], float)
    mu = np.array([0.5, 0.7])
    sol = np.array([0.0152695, 0.0073010, 0.0022325, 0.0, 0.0, 0.0])
    # uniform 4-dof layout: body 1 padded with two inert dofs (zero Jacobian, zero inverse mass)
    ndof = 4
    minv = np.zeros((2, ndof, ndof))
    minv[0] = np.linalg.inv(M0)
    minv[1, :2, :2] = np.linalg.inv(M1)
    HA = np.zeros((2, 3, ndof))
    HB = np.zeros((2, 3, ndof))
    HA[0] = H00
    HB[0, :, :2] = H01
    HA[1] = H10
    objA = [0, 0]
    objB = [1, -1]
    fpad = np.zeros(2 * ndof)
    fpad[:4] = f[:4]
    fpad[4:6] = f[4:6]
    # W = H M^-1 H^T, b = w - H M^-1 f (tests/GaussSeidel.cpp:23-27)
    Hd = np.zeros((6, 6))
    Hd[0:3, 0:4] = H00
    Hd[0:3, 4:6] = H01
    Hd[3:6, 0:4] = H10
    Minv = np.zeros((6, 6))
    Minv[:4, :4] = np.linalg.inv(M0)
    Minv[4:, 4:] = np.linalg.inv(M1)
    Wd = Hd @ Minv @ Hd.T
    b = w - Hd @ (Minv @ f)
    return {
        "source": "tests/SmallFrictionPb.hpp:18-67; tests/GaussSeidel.cpp:19-65; tests/ProjectedGradient.cpp:16-61",
        "dofs": dofs, "ndof_padded": ndof,
        "minv": minv.tolist(), "objA": objA, "objB": objB, "HA": HA.tolist(), "HB": HB.tolist(),
        "f_padded": fpad.tolist(), "w": w.tolist(), "mu": mu.tolist(), "sol": sol.tolist(),
        "W_dense": Wd.tolist(), "b": b.tolist(),
        "sol_rel_tol": 1e-4, "res_tol": 1e-8,
    }


def block_mv_symmetric():
    """tests/BlockMV.cpp:193-296 — 3x3-block symmetric matrix, lower storage."""
    ones = np.ones((3, 3))
    sec = np.array([[2, 0, 0], [2, 2, 0], [2, 2, 2]], float)
    blocks = [(0, 0, ones), (1, 0, sec), (2, 2, 3 * ones)]
    rowptr = [0, 1, 2, 3]
    col = [0, 0, 2]
    val = np.concatenate([b[2].reshape(-1) for b in blocks])
    return {
        "source": "tests/BlockMV.cpp:193-296",
        "rowptr": rowptr, "col": col, "val": val.tolist(),
        "rhs": [1.0] * 9,
        "expected_product": [9, 7, 5, 2, 4, 6, 9, 9, 9],
        "expected_split_row": [6, 4, 2, 2, 4, 6, 0, 0, 0],
    }


def polynomial():
    """tests/Polynomial.cpp:17-94 — quadratic roots and 3D SOC local quartic cases."""
    return {
        "source": "tests/Polynomial.cpp:17-94",
        "quadratic": [
            {"coeffs": [-1, 0], "filter": 0, "roots": [-1.0, 1.0]},
            {"coeffs": [-1, 0], "filter": 2, "roots": [1.0]},
            {"coeffs": [-1, 0], "filter": 1, "roots": [-1.0]},
            {"coeffs": [1, 0], "filter": 0, "roots": []},
            {"coeffs": [1, -2], "filter": 0, "roots": [1.0, 1.0]},
        ],
        "soc_quartic": [
            {"W": [0.01344, -9.421e-07, 0.001486, -9.421e-07, 0.1061, 0.0001733, 0.001486, 0.0001733, 0.001442],
             "b": [-0.1458, -0.2484, -0.1515], "mu": 0.6},
            {"W": [0.4, 0, 0, 0, 0.9, 0, 0, 0, 0.9], "b": [0, 0, 0.542629], "mu": 0.8},
            {"W": [0.4, 0, 0, 0, 1.4, 0, 0, 0, 1.4], "b": [-0.128762, 3.21747e-16, 14.5114], "mu": 0.8},
        ],
        "soc_quartic_checks": {"res_below": 1e-24, "complementarity_below": 1e-12},
    }


def projection():
    """tests/ProjectedGradient.cpp:85-108 — SOC projections, mu = (0.5, 3)."""
    return {
        "source": "tests/ProjectedGradient.cpp:85-108",
        "cases": [
            {"mu": 0.5, "x": [2, 0, 1], "expected": [2, 0, 1], "exact": True},
            {"mu": 3.0, "x": [1, 3, 0], "expected": [1, 3, 0], "exact": True},
            {"mu": 0.5, "x": [1, 3, 0], "expected": [2, 1, 0], "exact": False},
            {"mu": 0.5, "x": [-1, 7, 0], "expected": [2, 1, 0], "exact": False},
            {"mu": 3.0, "x": [-1, 0.3, 0], "expected": [0, 0, 0], "exact": False},
        ],
    }


def permutation():
    """tests/SparseBlock.cpp:464-498 — P W P^T on a symmetric matrix whose block (i, j) carries (i + j)."""
    return {
        "source": "tests/SparseBlock.cpp:464-498",
        "perm": [3, 1, 4, 2, 0, 7, 6, 5],
    }


def sparse_product():
    """tests/SparseBlock.cpp:16-60 — H H^T of a 3x4-block matrix: diagonal block (2,2) == 136, symmetry."""
    sample = np.array([1, 2, 3, 4, 3, 2, 1, 0, 1, 2, 3, 4], float).reshape(3, 4)
    return {
        "source": "tests/SparseBlock.cpp:16-60",
        "blocks": {"0,1": np.ones((3, 4)).tolist(), "1,0": sample.tolist(), "2,0": (3 * np.ones((3, 4))).tolist(),
                   "2,1": (5 * np.ones((3, 4))).tolist()},
        "diag2_value": 136.0,
    }


def main():
    out = {
        "small_friction_pb": small_friction_pb(),
        "block_mv_symmetric": block_mv_symmetric(),
        "polynomial": polynomial(),
        "projection": projection(),
        "permutation": permutation(),
        "sparse_product": sparse_product(),
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_fixtures.json")
    with open(path, "w") as fh:
        json.dump(out, fh, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
