"""Parallel driver of the oracle's Trotter sweeps (test infrastructure only).

The bonds of one sweep (all odd or all even links) touch disjoint Gammas and
Lambdas, so they are independent.  :class:`SweepPool` runs them on a pool of
spawned host processes, each calling :func:`oracle.two_site_op` or
:func:`oracle.two_site_op_nc` -- the functions ``oracle.trotter_step`` and
``oracle.trotter_step_nc`` call one bond after another, in the sweep order and
with the gate choice of ``TrotterStep2ndOrder`` / ``TrotterStep5thOrder`` and
their NC twins (VidalCore_v_2.0/propagation_module.f90:82-114, 200-252,
956-1018).  The result equals the sequential step's; only the order in which the
truncation errors are summed differs.

Gammas travel to the workers trimmed to their nonzero corner (rows and columns
that are entirely zero are dropped and restored as zeros on arrival), which keeps
a number-conserving chain at chi = 512 and low Schmidt rank cheap to ship.  Only
tests and the CPU legs of bench.py use this module; the product path never does.
"""
from __future__ import annotations

import multiprocessing as mp
import os

import numpy as np


def _trim(g):
    """(corner, chi): g[:ra, :, :rb] with every entry outside it zero."""
    rows = np.nonzero(np.any(g != 0, axis=(1, 2)))[0]
    cols = np.nonzero(np.any(g != 0, axis=(0, 1)))[0]
    ra = int(rows[-1]) + 1 if len(rows) else 0
    rb = int(cols[-1]) + 1 if len(cols) else 0
    return np.asfortranarray(g[:ra, :, :rb]), g.shape[0]


def _untrim(t):
    corner, chi = t
    g = np.zeros((chi, corner.shape[1], chi), dtype=np.complex128, order="F")
    g[: corner.shape[0], :, : corner.shape[2]] = corner
    return g


def _dense_bond(job):
    from oracle import oracle as O

    g1, g2, l0, l1, l2, op = job
    r = O.two_site_op(_untrim(g1), _untrim(g2), l0, l1, l2, op)
    return _trim(r[0]), _trim(r[1]), r[2], r[3]


def _nc_bond(job):
    from oracle import oracle as O

    g1, g2, l0, l1, l2, op, ll0, ll1, lr1, lr2, tot_num, max_filling = job
    r = O.two_site_op_nc(_untrim(g1), _untrim(g2), l0, l1, l2, op, ll0, ll1, lr1, lr2, tot_num,
                         max_filling)
    return _trim(r[0]), _trim(r[1]), r[2], r[3], r[4], r[5]


def _sweeps(order, L):
    """(links, gate index of each link) of every sweep of one step: 2nd order odd,
    even, odd with gate `link`; Forest-Ruth seven sweeps, odd first, with gate
    2 (link - 1) + (1, 1, 2, 2, 2, 1, 1)[sweep]."""
    if order == 2:
        pick = None
        n = 3
    elif order == 5:
        pick = (1, 1, 2, 2, 2, 1, 1)
        n = 7
    else:
        raise ValueError("order must be 2 or 5")
    out = []
    for s in range(n):
        links = list(range(1 if s % 2 == 0 else 2, L, 2))
        gates = [k if pick is None else 2 * (k - 1) + pick[s] for k in links]
        out.append((links, gates))
    return out


class SweepPool:
    """``with SweepPool() as P: P.trotter_step(gammas, lambdas, gates, order)``;
    the lists are updated in place, as by ``oracle.trotter_step``."""

    def __init__(self, processes=None):
        self.processes = processes or os.cpu_count() or 1

    def __enter__(self):
        os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")  # one LAPACK thread per worker
        self.pool = mp.get_context("spawn").Pool(self.processes)
        return self

    def __exit__(self, *exc):
        self.pool.close()
        self.pool.join()

    def trotter_step(self, gammas, lambdas, gates, order=2):
        L = len(gammas)
        tot = 0.0
        for links, gidx in _sweeps(order, L):
            jobs = [(_trim(gammas[k - 1]), _trim(gammas[k]), lambdas[k - 1], lambdas[k], lambdas[k + 1],
                     gates[g - 1]) for k, g in zip(links, gidx)]
            for k, (g1, g2, l1, te) in zip(links, self.pool.map(_dense_bond, jobs)):
                gammas[k - 1], gammas[k], lambdas[k] = _untrim(g1), _untrim(g2), l1
                tot += te
        return tot

    def trotter_step_nc(self, gammas, lambdas, label_left, label_right, gates, tot_num, max_filling, order=2):
        L = len(gammas)
        tot = 0.0
        for links, gidx in _sweeps(order, L):
            jobs = [(_trim(gammas[k - 1]), _trim(gammas[k]), lambdas[k - 1], lambdas[k], lambdas[k + 1],
                     gates[g - 1], label_left[k - 1], label_left[k], label_right[k], label_right[k + 1],
                     tot_num, max_filling) for k, g in zip(links, gidx)]
            for k, (g1, g2, l1, ll1, lr1, te) in zip(links, self.pool.map(_nc_bond, jobs)):
                gammas[k - 1], gammas[k], lambdas[k] = _untrim(g1), _untrim(g2), l1
                label_left[k], label_right[k] = ll1, lr1
                tot += te
        return tot
