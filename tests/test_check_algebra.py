"""The lane-split algebra of the FP32 accuracy check (csrc/batch.cu:
check_mode), restated in complex128 and compared with the serial recursion.

The check re-solves a sampled mode of the backward invariant-imbedding
recursion R_i = (a_i R_{i+1} - b_i) / (a_i - c_i R_{i+1}) (the sweep of
src/bldfm/solver.py:307-374 solved from the top radiation condition) with
the flux product Q(j) = prod_{i < j} (c_i R_i + a_i) below the highest output
level jm.  Split over 32 lanes: each lane composes the Moebius matrices
A_i = [[a, -b], [-c, a]] of its run of levels in two halves at
s = clamp(jm, lo, hi) with the det product of the lower half, a suffix scan
gives the ratio at the top of each run, and the lane's flux factors follow
without a division per level from f_i = det A_i D_{i+1} / D_i (homogeneous
v_i = A_i v_{i+1}, v = (N, D)).  Output levels below s take a second pass.
No GPU: the restatement pins the formulas the kernel implements."""

import numpy as np


def serial(a, b, c, RL, jm):
    L = len(a)
    R = np.empty(L + 1, complex)
    R[L] = RL
    for i in range(L - 1, -1, -1):
        R[i] = (a[i] * R[i + 1] - b[i]) / (a[i] - c[i] * R[i + 1])
    Q = np.ones(L + 1, complex)
    for j in range(1, L + 1):
        Q[j] = Q[j - 1] * ((c[j - 1] * R[j - 1] + a[j - 1]) if j - 1 < jm else 1.0)
    return R, Q


def lane_split(a, b, c, RL, jm, outs, nl=32):
    L = len(a)

    def A(i):
        return np.array([[a[i], -b[i]], [-c[i], a[i]]])

    lo = [k * L // nl for k in range(nl)]
    hi = [(k + 1) * L // nl for k in range(nl)]
    sp = [min(max(jm, lo[k]), hi[k]) for k in range(nl)]
    Ml, Mh, Det, M = [], [], [], []
    for k in range(nl):
        ml, mh, d = np.eye(2, dtype=complex), np.eye(2, dtype=complex), 1.0 + 0j
        for i in range(lo[k], hi[k]):
            if i < sp[k]:
                ml = ml @ A(i)
                d *= a[i] ** 2 - b[i] * c[i]
            else:
                mh = mh @ A(i)
        Ml.append(ml), Mh.append(mh), Det.append(d), M.append(ml @ mh)
    S, acc = [None] * nl, np.eye(2, dtype=complex)
    for k in range(nl - 1, -1, -1):
        acc = M[k] @ acc
        S[k] = acc

    def mob(m, R):
        return (m[0, 0] * R + m[0, 1]) / (m[1, 0] * R + m[1, 1])

    Rtop = [mob(S[k + 1], RL) if k < nl - 1 else RL for k in range(nl)]
    vs = [Mh[k] @ np.array([Rtop[k], 1.0]) for k in range(nl)]
    vlo = [Ml[k] @ vs[k] for k in range(nl)]
    F = [Det[k] * vs[k][1] / vlo[k][1] if sp[k] > lo[k] else 1.0 for k in range(nl)]
    P = np.cumprod([1.0] + F[:-1])
    res = {}
    for k in range(nl):
        for j in outs:
            if not (lo[k] <= j < hi[k] and j <= jm):
                continue
            if j == sp[k]:
                res[j] = (vs[k][0] / vs[k][1], P[k] * F[k])
            else:
                v, G = vs[k].copy(), 1.0 + 0j
                for i in range(sp[k] - 1, j - 1, -1):
                    v = A(i) @ v
                    G *= a[i] ** 2 - b[i] * c[i]
                res[j] = (v[0] / v[1], P[k] * Det[k] / G * v[1] / vlo[k][1])
    if jm == L and L in outs:
        res[L] = (RL, P[nl - 1] * F[nl - 1])
    return res


def test_lane_split_matches_serial_recursion():
    rng = np.random.default_rng(1)
    for trial in range(24):
        L = int(rng.integers(5, 240))
        h = rng.uniform(0.05, 0.4, L)
        K = rng.uniform(0.3, 3.0, L)
        x = rng.uniform(0.01, 0.8, L) + 1j * rng.uniform(-0.5, 0.5, L)  # -T h^2 / K
        T = -x * K / h**2
        a = 1 - 0.5 * h * h / K * T
        b = -h / K - h**3 / K**2 / 6.0 * T
        c = T * h - h**3 / K / 6.0 * T * T
        RL = 1.0 / (K[-1] * np.sqrt(-T[-1] / K[-1]))
        jm = int(rng.integers(0, L + 1))
        outs = sorted({jm, *map(int, rng.integers(0, jm + 1, 3))})
        R, Q = serial(a, b, c, RL, jm)
        res = lane_split(a, b, c, RL, jm, outs)
        assert sorted(res) == outs
        for j in outs:
            assert abs(res[j][0] - R[j]) <= 1e-12 * abs(R[j]), (trial, j)
            assert abs(res[j][1] - Q[j]) <= 1e-12 * abs(Q[j]), (trial, j)
