"""Algorithmic flop model of one COSX task, per grid point.

A task is one (grid point g, shell pair (a, b)) of the fused G kernel,
counted in the reference's orientation (bra = the larger shell index ish,
ket = jsh; gpu/sgx_k.py:165-400).  With L = la + lb, NA = 2 la + 1,
NB = 2 lb + 1, NCA/NCB the Cartesian counts and K = npi * npj primitive
pairs:

    flops = K * f_prim + npi * 2 NA NB NCA + (2 if ish == jsh else 4) NA NB
    f_prim = 11 + 14 (L + 1) + 3 [C(L+4, 4) - (L + 1)]
             + sum_{ca, cb} [n_t n_u + 3 n_t n_u n_v + 1] + 2 NCA NB NCB

n_t = i + i' + 1 (likewise u, v) for ca = (i, j, k), cb = (i', j', k').
The terms are: geometry and exponent (11), Boys by Horner (13 per order
plus 2) and R000 (1 per order), the McMurchie-Davidson R recurrence
(3 per entry beyond R000), the Hermite sum, the ket and bra contraction
transforms and the G contraction.  FMA = 2 flops; compensation (hi/lo)
work and screening are excluded.  The native library carries the same
formula (csrc/host_pairs.cpp model_flops) to count kept work inside the
kernels; tests check that both agree.
"""
from math import comb

import numpy as np

from pyscf_wb97mv_fast_gb300.basis import cart_components


def task_flops(la, lb, npi, npj, diag):
    L = la + lb
    NA, NB = 2 * la + 1, 2 * lb + 1
    ca = cart_components(la)
    cb = cart_components(lb)
    NCA, NCB = len(ca), len(cb)
    herm = 0
    for (i, j, k) in ca:
        for (ip, jp, kp) in cb:
            nt, nu, nv = i + ip + 1, j + jp + 1, k + kp + 1
            herm += nt * nu + 3 * nt * nu * nv + 1
    fprim = (11 + 14 * (L + 1) + 3 * (comb(L + 4, 4) - (L + 1)) + herm
             + 2 * NCA * NB * NCB)
    return (npi * npj * fprim + npi * 2 * NA * NB * NCA
            + (2 if diag else 4) * NA * NB)


def pair_flops_table(mol):
    """Model flops per grid point of every shell pair ish >= jsh of mol (all
    pairs, no magnitude cut; generally contracted shells split per column,
    as the kernels treat them)."""
    shells = []
    for sh in mol.shells:
        for _ in range(sh.nctr):
            shells.append((sh.l, sh.nprim))
    out = np.empty(len(shells) * (len(shells) + 1) // 2, dtype=np.int64)
    n = 0
    cache = {}
    for i, (li, pi) in enumerate(shells):
        for j in range(i + 1):
            lj, pj = shells[j]
            key = (li, lj, pi, pj, i == j)
            v = cache.get(key)
            if v is None:
                v = cache[key] = task_flops(li, lj, pi, pj, i == j)
            out[n] = v
            n += 1
    return out
