"""CPU restatement of the trajectory consumers, in numpy (test
infrastructure only: the oracle for siminf_gpu_trajectory_u/_v and
siminf_gpu_prevalence; only the test suite imports it).

U (and V) are flat arrays in the solver's column-major layout: column col
(replicate-major, then time) holds Nn blocks of Nc values.

- trajectory(M, Nn, stride, ncol, variables, id): SimInf_u_dense2df and
  SimInf_v_dense2df (src/misc/SimInf_trajectory.c:566-620, 652-706): per
  one-based variable, the values of the selected nodes, rows ordered by
  column, then node.
- prevalence(U, Nn, Nc, ncol, cases, population, level, condition, id):
  calculate_prevalence (R/prevalence.R:72-96) -- sums of the case and
  population compartments per node (sum_compartments, :24-38), both
  multiplied by the condition (:78-82, evaluated per node and column as
  evaluate_condition does, :40-68), then colSums of the counts (level 1),
  of the counts > 0 (level 2), or the per-node quotient (level 3).  The
  condition is a Python function of the compartments' integer arrays, so it
  shares nothing with the device path's formula compiler.

Parity is pinned against the reference's own tests: tests/prevalence.R:41-85
(a 3-node SIR trajectory and its level-1 prevalences with and without
conditions and an index) and tests/trajectory.R:28-70 (U = 1:180 and 1:360
over 6 nodes, one and two replicates).
"""
import numpy as np


def _blocks(M, Nn, stride, ncol, id=None):
    X = np.asarray(M).reshape(ncol, Nn, stride)
    if id is not None:
        X = X[:, np.asarray(id, dtype=np.int64) - 1, :]
    return X


def trajectory(M, Nn, stride, ncol, variables, id=None):
    X = _blocks(M, Nn, stride, ncol, id)
    return np.stack([X[:, :, v - 1].reshape(-1) for v in variables])


def prevalence(U, Nn, Nc, ncol, cases, population, level=1, condition=None, id=None,
               names=None):
    X = _blocks(U, Nn, Nc, ncol, id).astype(np.int64)
    cmask = np.array([(cases >> c) & 1 for c in range(Nc)], dtype=np.int64)
    pmask = np.array([(population >> c) & 1 for c in range(Nc)], dtype=np.int64)
    num = (X * cmask).sum(axis=2)
    den = (X * pmask).sum(axis=2)
    if condition is not None:
        k = np.asarray(condition(**{names[c]: X[:, :, c] for c in range(Nc)}), dtype=bool)
        num = num * k
        den = den * k
    with np.errstate(divide="ignore", invalid="ignore"):
        if level == 1:
            return num.sum(axis=1) / den.sum(axis=1)
        if level == 2:
            return (num > 0).sum(axis=1) / (den > 0).sum(axis=1)
        return num / den
