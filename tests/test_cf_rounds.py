"""The parallel restatement of the reference's C/F splitting that the GPU
kernels (afepack_gb300/csrc/coarsen.cu) implement, checked on the CPU against
the oracle's sequential Project (src/AMGSolver.cpp:18-126) on every level of
small hierarchies.

Pass 1 is computed in rounds (a row is F once a lower C row holds it as a
strong neighbour, C once every such row is F); pass 2 decides the candidates
(rows that would be promoted against the pass-1 C points alone) once their
candidate strong neighbours below them are decided.  Both give the
sequential sweeps' flags exactly."""
import numpy as np
import pytest

import oracle as O


def _strength(rp, ci, v, alpha=0.25):
    n = len(rp) - 1
    av = np.abs(v)
    offd = np.ones(len(ci), bool)
    offd[rp[:-1][np.diff(rp) > 0]] = False
    beta = np.zeros(n)
    for i in range(n):
        s = av[rp[i] + 1:rp[i + 1]]
        beta[i] = (s.max() if s.size else 0.0) * alpha
    row = np.repeat(np.arange(n), np.diff(rp))
    strong = offd & ~(av < beta[row])
    return beta, row, strong


def _pass1(rp, ci, v):
    n = len(rp) - 1
    _, row, strong = _strength(rp, ci, v)
    m = strong & (ci > row)          # row j holds i = ci strongly, j < i
    src, dst = row[m], ci[m]
    st = np.zeros(n, np.int8)
    rounds = 0
    while (st == 0).any():
        rounds += 1
        s = st[src]
        any_c = np.zeros(n, bool)
        np.logical_or.at(any_c, dst, s == -1)
        pend = np.zeros(n, bool)
        np.logical_or.at(pend, dst, s == 0)
        u = st == 0
        st = st.copy()
        st[u & any_c] = 1
        st[u & ~any_c & ~pend] = -1
        assert rounds <= n
    return st


def _pass2(rp, ci, v, st1):
    n = len(rp) - 1
    beta, _, strong = _strength(rp, ci, v)
    rows = [ci[rp[i] + 1:rp[i + 1]] for i in range(n)]
    srows = [ci[rp[i] + 1:rp[i + 1]][strong[rp[i] + 1:rp[i + 1]]] for i in range(n)]
    c1 = st1 == -1

    def promote(i, prom):
        s = srows[i]
        dep = set(s[c1[s] | (prom[s] & (s < i))].tolist())
        return any(not c1[k] and not dep.intersection(rows[k].tolist()) for k in s if k > i)

    none = np.zeros(n, bool)
    cand = np.zeros(n, bool)
    for i in np.nonzero(st1 == 1)[0]:
        cand[i] = promote(i, none)
    done = ~cand
    prom = np.zeros(n, bool)
    while not done.all():
        nd, npr = done.copy(), prom.copy()
        for i in np.nonzero(~done)[0]:
            s = srows[i]
            if done[s[(s < i) & cand[s]]].all():
                npr[i] = promote(i, prom & done)
                nd[i] = True
        done, prom = nd, npr
    flag = st1.copy()
    flag[prom] = -1
    return flag


@pytest.mark.parametrize("make", ["2d_p1_48", "3d_p1_10", "2d_p2_12"])
def test_round_restatement_matches_sequential_project(make):
    from afepack_gb300 import workloads as W
    wl = {"2d_p1_48": lambda: W.poisson2d_p1(48), "3d_p1_10": lambda: W.poisson3d_p1(10),
          "2d_p2_12": lambda: W.elliptic2d_p2(12)}[make]()
    K, _ = O.assemble(wl.space, wl.acc_stiff, wl.acc_mass, wl.coef)
    O.apply_dirichlet(K, np.zeros(K.shape[0]), wl.space.dof_bmark != 0)
    A, levels = K, 0
    while A.shape[0] > 50:
        rp, ci, v = A.rowptr.astype(np.int64), A.cols.astype(np.int64), A.vals
        flag = _pass2(rp, ci, v, _pass1(rp, ci, v))
        P, cf = O.project(A)
        assert np.array_equal(flag, cf), (make, levels)
        A = O.rap(P, A)
        levels += 1
        if P.shape[0] == P.shape[1]:
            break
    assert levels >= 2
