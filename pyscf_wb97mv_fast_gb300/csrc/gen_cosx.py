"""Generates csrc/generated/cosx_classes.cuh: one straight-line device
function per shell-pair class (la >= lb, la <= 3) of the fused COSX kernel.

For one task (shell pair A, B; one grid point g per thread) it adds

    G_B[nu] += sum_mu A^g_{mu nu} F_A[mu]        (always)
    G_A[mu] += sum_nu A^g_{mu nu} F_B[nu]        (A != B)

without forming A: F is first taken to the Cartesian components of each
shell (f0 = c2s F_A, h0 = c2s F_B; s/p normalisations are folded into the
primitive prefactor), then for every primitive pair

    R^{(n)}_000 = c_n F_n(T),  c_n = C_a C_b K_AB 2 pi / p sqrt(theta)
                                     (-2 p theta)^n          (folded, hi+lo)
    R_tuv       McMurchie-Davidson recurrence, in place, levels L .. 0
    Ac[ca, cb]  = sum_t Ex sum_u Ey sum_v Ez R_tuv
    Y[cb]      += f0[ca] Ac[ca, cb],   X[ca] += Ac[ca, cb] h0[cb]

and G_B += c2s^T Y at the end of the task.  The bra side is shared by a
run of consecutive tasks with the same shell A (pairs are ordered by
(A, B) within a class): f0 is formed once per run (cosx_begin) and X is
carried across the run and added to G_A once (cosx_end).  The recurrence
and the
Hermite sum are the reference's math (pyscf_wb97mv_fast/gpu/sgx_k.py:
200-307, gpu/shellpairs.py:447-485); the order of contraction (F first,
no A block, no per-primitive contraction matrices) is this generator's.
Constants of the d/f spherical transforms are applied as
fmaf(c_hi, x, c_lo * x) (one rounding of the compensated product,
gpu/int3c1e.py:17-31).

Run as a script (or import and call ``write()``); ``build()`` of the
package runs it before compiling.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from pyscf_wb97mv_fast_gb300.basis import cart2sph, cart_components  # noqa

LMAX = 3


def class_id(la, lb):
    return la * (la + 1) // 2 + lb


def classes():
    return [(la, lb) for la in range(LMAX + 1) for lb in range(la + 1)]


def e_entries(la, lb):
    """Packed (i, i', t) per axis, E^{00}_0 excluded (it is 1)."""
    out = []
    for i in range(la + 1):
        for j in range(lb + 1):
            for t in range(i + j + 1):
                if i == 0 and j == 0:
                    continue
                out.append((i, j, t))
    return out


def e_stride(la, lb):
    n = 3 * len(e_entries(la, lb))
    return (n + 3) // 4 * 4


def hilo(c):
    hi = np.float32(c)
    lo = np.float32(np.float64(c) - np.float64(hi))
    return hi, lo


def flit(x):
    """C float literal that round-trips exactly."""
    x = np.float32(x)
    if x == 0:
        return '0.0f'
    return '%.9ef' % float(x)


def rname(t, u, v):
    return 'r_%d_%d_%d' % (t, u, v)


def gen_recurrence(L, lines, ind, packed=False):
    """In-place R recurrence over levels n = L .. 0 (only t+u+v <= L-n).
    packed: the same operations on float2 (two grid points per lane)."""
    def mul(d, a):
        return ('mul2(%s, %s)' if packed else '%s * %s') % (d, a)

    def step(d, a, c, b):
        if not packed:
            return 'fmaf(%s, %s, %s * %s)' % (d, a, flit(c), b)
        # c * b with c = 1 is b exactly (the scalar form's compiler folds it)
        cb = b if c == 1 else 'mul2(bc2(%s), %s)' % (flit(c), b)
        return 'fma2(%s, %s, %s)' % (d, a, cb)

    for n in range(L, -1, -1):
        m = L - n
        if m >= 1:
            # t >= 1 entries: for each (u, v), t descending
            for u in range(m):
                for v in range(m - u):
                    for t in range(m - u - v, 0, -1):
                        if t == 1:
                            expr = mul('dx', rname(0, u, v))
                        else:
                            expr = step('dx', rname(t - 1, u, v), t - 1,
                                        rname(t - 2, u, v))
                        lines.append('%s%s = %s;' % (ind, rname(t, u, v), expr))
            # t = 0, u >= 1
            for v in range(m):
                for u in range(m - v, 0, -1):
                    if u == 1:
                        expr = mul('dy', rname(0, 0, v))
                    else:
                        expr = step('dy', rname(0, u - 1, v), u - 1, rname(0, u - 2, v))
                    lines.append('%s%s = %s;' % (ind, rname(0, u, v), expr))
            # t = u = 0, v >= 1
            for v in range(m, 0, -1):
                if v == 1:
                    expr = mul('dz', rname(0, 0, 0))
                else:
                    expr = step('dz', rname(0, 0, v - 1), v - 1, rname(0, 0, v - 2))
                lines.append('%s%s = %s;' % (ind, rname(0, 0, v), expr))
        lines.append('%s%s = R000_%d;' % (ind, rname(0, 0, 0), n))


def ename(ax, i, j, t):
    return 'e%s_%d_%d_%d' % ('xyz'[ax], i, j, t)


def gen_hermite(la, lb, ca_c, cb_c, ind, lines, tag, packed=False):
    """s = sum_t Ex sum_u Ey sum_v Ez R_tuv for one (ca, cb); returns the
    variable holding it.  packed: float2 operations, the E values read
    from their broadcast pairs B<name>."""
    (i, j, k) = ca_c
    (ip, jp, kp) = cb_c
    ty = 'float2' if packed else 'float'

    def mul(e, r):
        return ('mul2(B%s, %s)' if packed else '%s * %s') % (e, r)

    def fma(e, r, acc):
        return ('fma2(B%s, %s, %s)' if packed else 'fmaf(%s, %s, %s)') % (e, r, acc)

    s_terms = []
    for t in range(i + ip + 1):
        u_terms = []
        for u in range(j + jp + 1):
            # z sum
            if k == 0 and kp == 0:
                zexpr = rname(t, u, 0)
            else:
                acc = None
                for v in range(k + kp + 1):
                    e = ename(2, k, kp, v)
                    acc = (mul(e, rname(t, u, v)) if acc is None
                           else fma(e, rname(t, u, v), acc))
                zexpr = acc
            if j == 0 and jp == 0:
                u_terms.append(zexpr)
            else:
                u_terms.append((ename(1, j, jp, u), zexpr))
        # combine u terms
        if j == 0 and jp == 0:
            yexpr = u_terms[0]
        else:
            acc = None
            for (e, z) in u_terms:
                zv = 'z%s_%d_%d' % (tag, t, len(lines))
                lines.append('%sconst %s %s = %s;' % (ind, ty, zv, z))
                acc = mul(e, zv) if acc is None else fma(e, zv, acc)
            yexpr = acc
        if i == 0 and ip == 0:
            s_terms.append(yexpr)
        else:
            s_terms.append((ename(0, i, ip, t), yexpr))
    if i == 0 and ip == 0:
        sexpr = s_terms[0]
    else:
        acc = None
        for (e, y) in s_terms:
            yv = 'y%s_%d' % (tag, len(lines))
            lines.append('%sconst %s %s = %s;' % (ind, ty, yv, y))
            acc = mul(e, yv) if acc is None else fma(e, yv, acc)
        sexpr = acc
    sv = 's%s' % tag
    lines.append('%sconst %s %s = %s;' % (ind, ty, sv, sexpr))
    return sv


def gen_transform_in(l, src, dst, ind, lines):
    """dst[c] = sum_mu c2s[c, mu] src[mu] (compensated), l >= 2; identity
    for l <= 1 (normalisation folded into the prefactor)."""
    nc = (l + 1) * (l + 2) // 2
    if l <= 1:
        for c in range(nc):
            lines.append('%sconst float %s%d = %s%d;' % (ind, dst, c, src, c))
        return
    c2s = cart2sph(l)
    for c in range(nc):
        terms = []
        for mu in range(2 * l + 1):
            v = c2s[c, mu]
            if abs(v) < 1e-15:
                continue
            hi, lo = hilo(v)
            terms.append('fmaf(%s, %s%d, %s * %s%d)' % (
                flit(hi), src, mu, flit(lo), src, mu))
        expr = ' + '.join(terms) if terms else '0.0f'
        lines.append('%sconst float %s%d = %s;' % (ind, dst, c, expr))


def gen_transform_out(l, src, dst, ind, lines):
    """dst[mu] = sum_c c2s[c, mu] src[c] (compensated), l >= 2."""
    if l <= 1:
        for c in range(2 * l + 1):
            lines.append('%sconst float %s%d = %s%d;' % (ind, dst, c, src, c))
        return
    c2s = cart2sph(l)
    nc = (l + 1) * (l + 2) // 2
    for mu in range(2 * l + 1):
        terms = []
        for c in range(nc):
            v = c2s[c, mu]
            if abs(v) < 1e-15:
                continue
            hi, lo = hilo(v)
            terms.append('fmaf(%s, %s%d, %s * %s%d)' % (
                flit(hi), src, c, flit(lo), src, c))
        expr = ' + '.join(terms) if terms else '0.0f'
        lines.append('%sconst float %s%d = %s;' % (ind, dst, mu, expr))


def gen_begin(la):
    """f0 = c2s^T F_A of the run's A shell (F_A loaded by the caller)."""
    na = 2 * la + 1
    nca = (la + 1) * (la + 2) // 2
    lines = ['template<> __device__ __forceinline__ void cosx_begin<%d>(' % la,
             '    const float* fa_in, float* f0)',
             '{']
    I = '    '
    for mu in range(na):
        lines.append(I + 'const float fa%d = fa_in[%d];' % (mu, mu))
    gen_transform_in(la, 'fa', 'c', I, lines)
    for c in range(nca):
        lines.append(I + 'f0[%d] = c%d;' % (c, c))
    lines.append('}')
    return '\n'.join(lines)


def gen_end(la):
    """G_A = c2s^T X at the end of a run: a plain store into the class's
    partial-G buffer (no other task of the class writes the row before)."""
    na = 2 * la + 1
    nca = (la + 1) * (la + 2) // 2
    lines = ['template<> __device__ __forceinline__ void cosx_end<%d>(' % la,
             '    float* __restrict__ Gp, const int ga0, const int ld,',
             '    const bool ok, const float* Xa)',
             '{']
    I = '    '
    for c in range(nca):
        lines.append(I + 'const float X%d = Xa[%d];' % (c, c))
    gen_transform_out(la, 'X', 'gv', I, lines)
    lines.append(I + 'if (!ok) return;')
    for mu in range(na):
        lines.append(I + 'Gp[(long long)(ga0 + %d) * ld] = gv%d;' % (mu, mu))
    lines.append('}')
    return '\n'.join(lines)


def n_om(la, lb):
    """float4 per primitive pair of the omega record a class reads: theta p
    and c_0..c_L (hi + lo), then the far-field float4 (K0 hi, K0 lo, r^2
    threshold)."""
    return 2 + (la + lb + 1) // 2


def pipe_e(la, lb):
    """Whether the Hermite E record is prefetched one primitive pair ahead
    (small records only: the prefetch doubles its registers)."""
    return e_stride(la, lb) // 4 <= 6 and (la + lb) >= 1


def rec_stride(la, lb):
    """float4 per primitive pair of a class's packed record: geo (P hi,
    P lo), the omega record's first n_om float4, the Hermite E block."""
    return 2 + n_om(la, lb) + e_stride(la, lb) // 4


def gen_rec(la, lb):
    """Per-class record of one primitive pair (geo, omega and, for small
    classes, E) and its loader: the task loop keeps the next pair's record
    in flight while it computes the current one.  m is class-local."""
    nom = n_om(la, lb)
    nvec = e_stride(la, lb) // 4 if pipe_e(la, lb) else 0
    mem = ['g0', 'g1'] + ['o%d' % q for q in range(nom)] + \
          ['e%d' % q for q in range(nvec)]
    lines = ['template<> struct CosxRec<%d, %d> {' % (la, lb),
             '    float4 %s;' % ', '.join(mem),
             '};',
             'template<bool FAR> __device__ __forceinline__ void cosx_rec_load(',
             '    const CosxArgs& A, const int m, CosxRec<%d, %d>& r)' % (la, lb),
             '{']
    I = '    '
    lines.append(I + 'const float4* __restrict__ q = A.rec[%d] + (long long)m * %d;'
                 % (class_id(la, lb), rec_stride(la, lb)))
    lines.append(I + 'r.g0 = __ldg(q);')
    lines.append(I + 'r.g1 = __ldg(q + 1);')
    for k in range(nom - 1):
        lines.append(I + 'r.o%d = __ldg(q + %d);' % (k, 2 + k))
    lines.append(I + 'r.o%d = __ldg(q + %d);' % (nom - 1, 1 + nom))
    for k in range(nvec):
        lines.append(I + 'r.e%d = __ldg(q + %d);' % (k, 2 + nom + k))
    lines.append('}')
    return '\n'.join(lines)


def gen_prim_body(la, lb, diag, rv, J, lines, far=True, stage=False):
    """Work of primitive pair m with its record in variable rv (a CosxRec,
    or with stage a pointer to the record in shared memory), for each of
    the PTS points of the lane: Boys, R recurrence, Hermite sums and the Y
    (and X) accumulation.  The record and E are shared by the points."""
    L = la + lb
    ca = cart_components(la)
    cb = cart_components(lb)
    ents = e_entries(la, lb)
    est = e_stride(la, lb)
    nom = n_om(la, lb)
    nvec = est // 4
    comp = 'xyzw'
    tuv = [(t, u, v) for t in range(L + 1) for u in range(L + 1 - t)
           for v in range(L + 1 - t - u)]
    if stage:
        lines.append(J + 'const float4 ph = %s[0], pl = %s[1];' % (rv, rv))
        for q in range(nom):
            lines.append(J + 'const float4 o%d = %s[%d];' % (q, rv, 2 + q))
    else:
        lines.append(J + 'const float4 ph = %s.g0, pl = %s.g1;' % (rv, rv))
        for q in range(nom):
            lines.append(J + 'const float4 o%d = %s.o%d;' % (q, rv, q))
    if ents:
        if stage:
            for q in range(nvec):
                lines.append(J + 'const float4 ev%d = %s[%d];' % (q, rv, 2 + nom + q))
        elif pipe_e(la, lb):
            for q in range(nvec):
                lines.append(J + 'const float4 ev%d = %s.e%d;' % (q, rv, q))
        else:
            lines.append(J + 'const float4* __restrict__ Em = A.rec[%d] + (long long)m * %d + %d;'
                         % (class_id(la, lb), rec_stride(la, lb), 2 + nom))
            for q in range(nvec):
                lines.append(J + 'const float4 ev%d = __ldg(Em + %d);' % (q, q))
        flat = []
        for ax in range(3):
            for (i, j, t) in ents:
                flat.append(ename(ax, i, j, t))
        while len(flat) % 4:
            flat.append(None)
        for q in range(nvec):
            for c in range(4):
                nm = flat[4 * q + c]
                if nm is not None:
                    lines.append(J + 'const float %s = ev%d.%s;' % (nm, q, comp[c]))
    if not far:
        # long-range omegas: T = theta p r^2 stays below 36 almost always,
        # so one warp vote selects the branch-free Taylor form for every
        # point; mixed warps take the far-field form where T >= 36
        of = 'o%d' % (nom - 1)
        lines.append(J + 'float dxv[PTS], dyv[PTS], dzv[PTS], r2v[PTS], R0[PTS][%d];' % (L + 1))
        lines.append(J + 'bool allnear = true;')
        lines.append(J + '#pragma unroll')
        lines.append(J + 'for (int p = 0; p < PTS; ++p) {')
        lines.append(J + '    dxv[p] = (ph.x - gxh[p]) + (pl.x - gxl[p]);')
        lines.append(J + '    dyv[p] = (ph.y - gyh[p]) + (pl.y - gyl[p]);')
        lines.append(J + '    dzv[p] = (ph.z - gzh[p]) + (pl.z - gzl[p]);')
        lines.append(J + '    r2v[p] = fmaf(dxv[p], dxv[p], fmaf(dyv[p], dyv[p], dzv[p] * dzv[p]));')
        lines.append(J + '    allnear = allnear && r2v[p] < %s.z;' % of)
        lines.append(J + '}')

        def near_n(ind, p):
            lines.append(ind + 'const float T = fmaf(o0.x, r2v[%s], o0.y * r2v[%s]);' % (p, p))
            lines.append(ind + 'float Fb[%d];' % (L + 1))
            lines.append(ind + 'boys_taylor<%d>(T, Fb, stab);' % L)
            for n in range(L + 1):
                fh = 2 + 2 * n
                fl = fh + 1
                ch = 'o%d.%s' % (fh // 4, comp[fh % 4])
                cl = 'o%d.%s' % (fl // 4, comp[fl % 4])
                lines.append(ind + 'R0[%s][%d] = fmaf(%s, Fb[%d], %s * Fb[%d]);'
                             % (p, n, ch, n, cl, n))

        lines.append(J + 'if (__all_sync(0xffffffffu, allnear)) {')
        lines.append(J + '    #pragma unroll')
        lines.append(J + '    for (int p = 0; p < PTS; ++p) {')
        near_n(J + '        ', 'p')
        lines.append(J + '    }')
        lines.append(J + '} else {')
        lines.append(J + '    #pragma unroll')
        lines.append(J + '    for (int p = 0; p < PTS; ++p) {')
        lines.append(J + '        if (r2v[p] >= %s.z) {' % of)
        lines.append(J + '            far_r000<%d>(r2v[p], %s.x, %s.y, R0[p]);' % (L, of, of))
        lines.append(J + '        } else {')
        near_n(J + '            ', 'p')
        lines.append(J + '        }')
        lines.append(J + '    }')
        lines.append(J + '}')
    else:
        of = 'o%d' % (nom - 1)          # far-field float4: K0 hi, K0 lo, thr
        # distances, then R000 for every point: the far-field form when the
        # whole warp is far (a uniform branch), else per point
        lines.append(J + 'float dxv[PTS], dyv[PTS], dzv[PTS], r2v[PTS];')
        lines.append(J + 'bool allfar = true, anyfar = false;')
        lines.append(J + '#pragma unroll')
        lines.append(J + 'for (int p = 0; p < PTS; ++p) {')
        lines.append(J + '    dxv[p] = (ph.x - gxh[p]) + (pl.x - gxl[p]);')
        lines.append(J + '    dyv[p] = (ph.y - gyh[p]) + (pl.y - gyl[p]);')
        lines.append(J + '    dzv[p] = (ph.z - gzh[p]) + (pl.z - gzl[p]);')
        lines.append(J + '    r2v[p] = fmaf(dxv[p], dxv[p], fmaf(dyv[p], dyv[p], dzv[p] * dzv[p]));')
        lines.append(J + '    const bool f = r2v[p] >= %s.z;' % of)
        lines.append(J + '    allfar = allfar && f;')
        lines.append(J + '    anyfar = anyfar || f;')
        lines.append(J + '}')
        lines.append(J + 'float R0[PTS][%d];' % (L + 1))

        def near(ind, p):
            lines.append(ind + 'const float T = fmaf(o0.x, r2v[%s], o0.y * r2v[%s]);' % (p, p))
            lines.append(ind + 'float Fb[%d];' % (L + 1))
            lines.append(ind + 'boys_taylor<%d>(T, Fb, stab);' % L)
            for n in range(L + 1):
                fh = 2 + 2 * n
                fl = fh + 1
                ch = 'o%d.%s' % (fh // 4, comp[fh % 4])
                cl = 'o%d.%s' % (fl // 4, comp[fl % 4])
                lines.append(ind + 'R0[%s][%d] = fmaf(%s, Fb[%d], %s * Fb[%d]);'
                             % (p, n, ch, n, cl, n))

        # uniform branches when the whole warp is far (T >= 36) or near; the
        # per-point branch only for mixed warps
        lines.append(J + 'if (__all_sync(0xffffffffu, allfar)) {')
        lines.append(J + '    #pragma unroll')
        lines.append(J + '    for (int p = 0; p < PTS; ++p)')
        lines.append(J + '        far_r000<%d>(r2v[p], %s.x, %s.y, R0[p]);' % (L, of, of))
        lines.append(J + '} else if (!__any_sync(0xffffffffu, anyfar)) {')
        lines.append(J + '    #pragma unroll')
        lines.append(J + '    for (int p = 0; p < PTS; ++p) {')
        near(J + '        ', 'p')
        lines.append(J + '    }')
        lines.append(J + '} else {')
        lines.append(J + '    #pragma unroll')
        lines.append(J + '    for (int p = 0; p < PTS; ++p) {')
        lines.append(J + '        if (r2v[p] >= %s.z) {' % of)
        lines.append(J + '            far_r000<%d>(r2v[p], %s.x, %s.y, R0[p]);' % (L, of, of))
        lines.append(J + '        } else {')
        near(J + '            ', 'p')
        lines.append(J + '        }')
        lines.append(J + '    }')
        lines.append(J + '}')
    lines.append(J + '#pragma unroll')
    lines.append(J + 'for (int p = 0; p < PTS; ++p) {')
    K = J + '    '
    lines.append(K + 'const float dx = dxv[p], dy = dyv[p], dz = dzv[p];')
    for n in range(L + 1):
        lines.append(K + 'const float R000_%d = R0[p][%d];' % (n, n))
    lines.append(K + 'float ' + ', '.join(rname(*x) for x in tuv) + ';')
    gen_recurrence(L, lines, K)
    for ia, cac in enumerate(ca):
        for ib, cbc in enumerate(cb):
            tag = '%d_%d' % (ia, ib)
            sv = gen_hermite(la, lb, cac, cbc, K, lines, tag)
            lines.append(K + 'Yv[p][%d] = fmaf(f0v[p][%d], %s, Yv[p][%d]);'
                         % (ib, ia, sv, ib))
            if not diag:
                lines.append(K + 'Xv[p][%d] = fmaf(%s, h0v[p][%d], Xv[p][%d]);'
                             % (ia, sv, ib, ia))
    lines.append(J + '}')


def gen_class(la, lb, diag, far, stage=False):
    nb = 2 * lb + 1
    nca = (la + 1) * (la + 2) // 2
    ncb = (lb + 1) * (lb + 2) // 2
    ents = e_entries(la, lb)
    lines = []
    I = '    '
    lines.append('template<int PTS> struct CosxTask<%d, %d, %s, PTS, %s, %s> {'
                 % (la, lb, 'true' if diag else 'false', 'true' if far else 'false',
                    'true' if stage else 'false'))
    lines.append('static __device__ __forceinline__ void run(')
    lines.append('    const CosxArgs& A, float* const* Gp, const int ld, const int gb0,')
    if stage:
        lines.append('    const float4* __restrict__ rp, const int npp, const bool* ok,')
    else:
        lines.append('    const int pp0, const int npp, const int nxt, const bool* ok,')
    lines.append('    const float* gxh, const float* gyh, const float* gzh,')
    lines.append('    const float* gxl, const float* gyl, const float* gzl,')
    lines.append('    const float4* __restrict__ stab, const float* f0,')
    if stage:
        lines.append('    const float* fb, float* Xa)')
    else:
        lines.append('    const float* fb, float* Xa, CosxRec<%d, %d>& rec)' % (la, lb))
    lines.append('{')
    lines.append(I + 'float f0v[PTS][%d], Yv[PTS][%d];' % (nca, ncb))
    if not diag:
        lines.append(I + 'float gbo[PTS][%d], h0v[PTS][%d], Xv[PTS][%d];'
                     % (nb, ncb, nca))
    lines.append(I + '#pragma unroll')
    lines.append(I + 'for (int p = 0; p < PTS; ++p) {')
    J = I * 2
    if not diag:
        # WB_COSX_GB_RED = 0: G_B read early (its latency overlaps the
        # primitive loop), added to and stored at the end
        lines.append('#if !WB_COSX_GB_RED')
        for nu in range(nb):
            lines.append(J + 'gbo[p][%d] = Gp[p][(long long)(gb0 + %d) * ld];'
                         % (nu, nu))
        lines.append('#endif')
        for nu in range(nb):
            lines.append(J + 'const float fb%d = fb[p * %d + %d];' % (nu, nb, nu))
        gen_transform_in(lb, 'fb', 'h0_', J, lines)
        for c in range(ncb):
            lines.append(J + 'h0v[p][%d] = h0_%d;' % (c, c))
        for c in range(nca):
            lines.append(J + 'Xv[p][%d] = Xa[p * %d + %d];' % (c, nca, c))
    for c in range(nca):
        lines.append(J + 'f0v[p][%d] = f0[p * %d + %d];' % (c, nca, c))
    for c in range(ncb):
        lines.append(J + 'Yv[p][%d] = 0.0f;' % c)
    lines.append(I + '}')
    if stage:
        # records staged in shared memory by the caller: one base address
        lines.append(I + '#pragma unroll 1')
        lines.append(I + 'for (int m = 0; m < npp; ++m) {')
        lines.append(J + 'const float4* __restrict__ q = rp + m * %d;' % rec_stride(la, lb))
        lines.append(J + '{')
        gen_prim_body(la, lb, diag, 'q', J + I, lines, far, stage=True)
        lines.append(J + '}')
        lines.append(I + '}')
    else:
        lines.append(I + 'const int pend = pp0 + npp;')
        # two register sets for the primitive-pair record (rec, rb) used in
        # turn: while one pair computes, the next one loads into the other set
        lines.append(I + 'CosxRec<%d, %d> rb;' % (la, lb))
        lines.append(I + 'int m = pp0;')
        lines.append(I + '#pragma unroll 1')
        lines.append(I + 'while (true) {')
        lines.append(J + 'cosx_rec_load<%s>(A, m + 1 < pend ? m + 1 : nxt, rb);'
                     % ('true' if far else 'false'))
        lines.append(J + '{')
        gen_prim_body(la, lb, diag, 'rec', J + I, lines, far)
        lines.append(J + '}')
        lines.append(J + 'if (++m == pend) { rec = rb; break; }')
        lines.append(J + 'cosx_rec_load<%s>(A, m + 1 < pend ? m + 1 : nxt, rec);'
                     % ('true' if far else 'false'))
        lines.append(J + '{')
        gen_prim_body(la, lb, diag, 'rb', J + I, lines, far)
        lines.append(J + '}')
        lines.append(J + 'if (++m == pend) break;')
        lines.append(I + '}')
    lines.append(I + '#pragma unroll')
    lines.append(I + 'for (int p = 0; p < PTS; ++p) {')
    if diag:
        # B = A: the ket contribution joins the run's bra accumulator, which
        # cosx_end transforms and stores once
        for c in range(ncb):
            lines.append(J + 'Xa[p * %d + %d] += Yv[p][%d];' % (nca, c, c))
    else:
        for c in range(ncb):
            lines.append(J + 'const float Y%d = Yv[p][%d];' % (c, c))
        gen_transform_out(lb, 'Y', 'gy', J, lines)
        lines.append(J + 'if (ok[p]) {')
        for nu in range(nb):
            lines.append('#if WB_COSX_GB_RED')
            lines.append(J + '    gb_add(Gp[p] + (long long)(gb0 + %d) * ld, gy%d);'
                         % (nu, nu))
            lines.append('#else')
            lines.append(J + '    Gp[p][(long long)(gb0 + %d) * ld] = gbo[p][%d] + gy%d;'
                         % (nu, nu, nu))
            lines.append('#endif')
        lines.append(J + '}')
        for c in range(nca):
            lines.append(J + 'Xa[p * %d + %d] = Xv[p][%d];' % (nca, c, c))
    lines.append(I + '}')
    lines.append('}')
    lines.append('};')
    return '\n'.join(lines)


def rec_stride2(la, lb):
    """float4 per primitive pair of a class's dual-omega packed record: geo,
    the two omegas' records (n_om float4 each), E."""
    return 2 + 2 * n_om(la, lb) + e_stride(la, lb) // 4


def gen_r000(la, lb, J, lines, of_prefix, near_first, slot, packed=False):
    """R0[slot][p][n] for every point from the distances r2v, with the
    omega record fields named <of_prefix><q>: warp-uniform all-far /
    all-near branches (the likelier one tested first), per point for mixed
    warps.  packed (PTS = 2): R0p[slot][n] float2 pairs, the all-far branch
    on both points at once (far_r000_v<L, float2>)."""
    L = la + lb
    nom = n_om(la, lb)
    comp = 'xyzw'
    o = lambda q: '%s%d' % (of_prefix, q)
    of = o(nom - 1)

    def dst(p, n):
        return ('R0p[%d][%d].%s' % (slot, n, 'xy'[int(p)]) if packed
                else 'R0[%d][p][%d]' % (slot, n))

    def near(ind, p='p'):
        lines.append(ind + 'const float T = fmaf(%s.x, r2v[%s], %s.y * r2v[%s]);'
                     % (o(0), p, o(0), p))
        lines.append(ind + 'float Fb[%d];' % (L + 1))
        lines.append(ind + 'boys_taylor<%d>(T, Fb, stab);' % L)
        for n in range(L + 1):
            fh = 2 + 2 * n
            fl = fh + 1
            ch = '%s.%s' % (o(fh // 4), comp[fh % 4])
            cl = '%s.%s' % (o(fl // 4), comp[fl % 4])
            lines.append(ind + '%s = fmaf(%s, Fb[%d], %s * Fb[%d]);'
                         % (dst(p, n), ch, n, cl, n))

    def far(ind, p='p'):
        if not packed:
            lines.append(ind + 'far_r000<%d>(r2v[p], %s.x, %s.y, R0[%d][p]);'
                         % (L, of, of, slot))
            return
        lines.append(ind + 'float Rt[%d];' % (L + 1))
        lines.append(ind + 'far_r000<%d>(r2v[%s], %s.x, %s.y, Rt);' % (L, p, of, of))
        for n in range(L + 1):
            lines.append(ind + '%s = Rt[%d];' % (dst(p, n), n))

    def far_all(ind):
        lines.append(ind + 'far_r000_v<%d, float2>(r2, %s.x, %s.y, R0p[%d]);'
                     % (L, of, of, slot))

    def per_point(ind, body):
        if packed:
            for p in range(2):
                lines.append(ind + '{')
                body(ind + '    ', str(p))
                lines.append(ind + '}')
        else:
            lines.append(ind + '#pragma unroll')
            lines.append(ind + 'for (int p = 0; p < PTS; ++p) {')
            body(ind + '    ')
            lines.append(ind + '}')

    def branch(kind, ind):
        if kind == 'far' and packed:
            far_all(ind)
        else:
            per_point(ind, far if kind == 'far' else near)

    lines.append(J + '{')
    K = J + '    '
    lines.append(K + 'bool allfar = true, allnear = true;')
    lines.append(K + '#pragma unroll')
    lines.append(K + 'for (int p = 0; p < PTS; ++p) {')
    lines.append(K + '    const bool f = r2v[p] >= %s.z;' % of)
    lines.append(K + '    allfar = allfar && f;')
    lines.append(K + '    allnear = allnear && !f;')
    lines.append(K + '}')
    first, second = (('allnear', 'near'), ('allfar', 'far')) if near_first else (('allfar', 'far'), ('allnear', 'near'))
    lines.append(K + 'if (__all_sync(0xffffffffu, %s)) {' % first[0])
    branch(first[1], K + '    ')
    lines.append(K + '} else if (__all_sync(0xffffffffu, %s)) {' % second[0])
    branch(second[1], K + '    ')
    lines.append(K + '} else {')

    def mixed(ind, p='p'):
        lines.append(ind + 'if (r2v[%s] >= %s.z) {' % (p, of))
        far(ind + '    ', p)
        lines.append(ind + '} else {')
        near(ind + '    ', p)
        lines.append(ind + '}')
    per_point(K + '    ', mixed)
    lines.append(K + '}')
    lines.append(J + '}')


def gen_prim_body_dual(la, lb, diag, J, lines, packed=False):
    """Dual-omega work of one primitive pair whose record is at q (shared
    memory): the distances once, then for each omega slot the R000 sources
    (slot 0: all-far tested first, slot 1: all-near first), the R
    recurrence, the Hermite sums and the Y (and X) accumulation.

    packed (PTS = 2): the distances, recurrence, Hermite sums and
    accumulations run on float2 pairs of the lane's two points, the same
    operations in the same order as the scalar body; the R000 sources
    (Boys function, far form, the warp votes) stay per point."""
    L = la + lb
    ca = cart_components(la)
    cb = cart_components(lb)
    ents = e_entries(la, lb)
    nom = n_om(la, lb)
    nvec = e_stride(la, lb) // 4
    comp = 'xyzw'
    tuv = [(t, u, v) for t in range(L + 1) for u in range(L + 1 - t)
           for v in range(L + 1 - t - u)]
    lines.append(J + 'const float4 ph = q[0], pl = q[1];')
    for w, pre in enumerate(('oa', 'ob')):
        for k in range(nom):
            lines.append(J + 'const float4 %s%d = q[%d];' % (pre, k, 2 + w * nom + k))
    if ents:
        for k in range(nvec):
            lines.append(J + 'const float4 ev%d = q[%d];' % (k, 2 + 2 * nom + k))
        flat = []
        for ax in range(3):
            for (i, j, t) in ents:
                flat.append(ename(ax, i, j, t))
        while len(flat) % 4:
            flat.append(None)
        for k in range(nvec):
            for c in range(4):
                nm = flat[4 * k + c]
                if nm is not None:
                    lines.append(J + 'const float %s = ev%d.%s;' % (nm, k, comp[c]))
                    if packed:
                        lines.append(J + 'const float2 B%s = bc2(%s);' % (nm, nm))
    if packed:
        # a - b as a + (-b) (exact), the grid's negated pairs made once per task
        lines.append(J + 'float r2v[PTS];')
        lines.append(J + 'float2 R0p[2][%d];' % (L + 1))
        for ax in 'xyz':
            lines.append(J + 'const float2 d%s = add2(add2(bc2(ph.%s), NG%sH), '
                         'add2(bc2(pl.%s), NG%sL));' % (ax, ax, ax.upper(), ax, ax.upper()))
        lines.append(J + 'const float2 r2 = fma2(dx, dx, fma2(dy, dy, mul2(dz, dz)));')
        lines.append(J + 'r2v[0] = r2.x;')
        lines.append(J + 'r2v[1] = r2.y;')
    else:
        lines.append(J + 'float dxv[PTS], dyv[PTS], dzv[PTS], r2v[PTS], R0[2][PTS][%d];' % (L + 1))
        lines.append(J + '#pragma unroll')
        lines.append(J + 'for (int p = 0; p < PTS; ++p) {')
        lines.append(J + '    dxv[p] = (ph.x - gxh[p]) + (pl.x - gxl[p]);')
        lines.append(J + '    dyv[p] = (ph.y - gyh[p]) + (pl.y - gyl[p]);')
        lines.append(J + '    dzv[p] = (ph.z - gzh[p]) + (pl.z - gzl[p]);')
        lines.append(J + '    r2v[p] = fmaf(dxv[p], dxv[p], fmaf(dyv[p], dyv[p], dzv[p] * dzv[p]));')
        lines.append(J + '}')
    # the common case of a full-range + long-range pair: slot a far and slot
    # b near for the whole warp -- one vote, both slots in one basic block
    ofa, ofb = 'oa%d' % (nom - 1), 'ob%d' % (nom - 1)
    lines.append(J + 'bool farnear = true;')
    lines.append(J + '#pragma unroll')
    lines.append(J + 'for (int p = 0; p < PTS; ++p)')
    lines.append(J + '    farnear = farnear && r2v[p] >= %s.z && r2v[p] < %s.z;' % (ofa, ofb))
    lines.append(J + 'if (__all_sync(0xffffffffu, farnear)) {')
    K = J + '    '

    def near_b(ind, p, dst):
        lines.append(ind + 'const float T = fmaf(ob0.x, r2v[%s], ob0.y * r2v[%s]);' % (p, p))
        lines.append(ind + 'float Fb[%d];' % (L + 1))
        lines.append(ind + 'boys_taylor<%d>(T, Fb, stab);' % L)
        for n in range(L + 1):
            fh = 2 + 2 * n
            fl = fh + 1
            ch = 'ob%d.%s' % (fh // 4, comp[fh % 4])
            cl = 'ob%d.%s' % (fl // 4, comp[fl % 4])
            lines.append(ind + '%s = fmaf(%s, Fb[%d], %s * Fb[%d]);'
                         % (dst(n), ch, n, cl, n))

    if packed:
        lines.append(K + 'far_r000_v<%d, float2>(r2, %s.x, %s.y, R0p[0]);' % (L, ofa, ofa))
        for p in range(2):
            lines.append(K + '{')
            near_b(K + '    ', str(p), lambda n, p=p: 'R0p[1][%d].%s' % (n, 'xy'[p]))
            lines.append(K + '}')
    else:
        lines.append(K + '#pragma unroll')
        lines.append(K + 'for (int p = 0; p < PTS; ++p) {')
        lines.append(K + '    far_r000<%d>(r2v[p], %s.x, %s.y, R0[0][p]);' % (L, ofa, ofa))
        near_b(K + '    ', 'p', lambda n: 'R0[1][p][%d]' % n)
        lines.append(K + '}')
    lines.append(J + '} else {')
    gen_r000(la, lb, K, lines, 'oa', False, 0, packed)
    gen_r000(la, lb, K, lines, 'ob', True, 1, packed)
    lines.append(J + '}')
    lines.append(J + '#pragma unroll')
    lines.append(J + 'for (int w = 0; w < 2; ++w) {')
    if packed:
        K = J + '    '
        for n in range(L + 1):
            lines.append(K + 'const float2 R000_%d = R0p[w][%d];' % (n, n))
        lines.append(K + 'float2 ' + ', '.join(rname(*x) for x in tuv) + ';')
        gen_recurrence(L, lines, K, packed=True)
        for ia, cac in enumerate(ca):
            for ib, cbc in enumerate(cb):
                tag = '%d_%d' % (ia, ib)
                sv = gen_hermite(la, lb, cac, cbc, K, lines, tag, packed=True)
                lines.append(K + 'Yp[w][%d] = fma2(f0p[%d], %s, Yp[w][%d]);'
                             % (ib, ia, sv, ib))
                if not diag:
                    lines.append(K + 'Xp[w][%d] = fma2(%s, h0p[%d], Xp[w][%d]);'
                                 % (ia, sv, ib, ia))
        lines.append(J + '}')
        return
    lines.append(J + '#pragma unroll')
    lines.append(J + 'for (int p = 0; p < PTS; ++p) {')
    K = J + '    '
    lines.append(K + 'const float dx = dxv[p], dy = dyv[p], dz = dzv[p];')
    for n in range(L + 1):
        lines.append(K + 'const float R000_%d = R0[w][p][%d];' % (n, n))
    lines.append(K + 'float ' + ', '.join(rname(*x) for x in tuv) + ';')
    gen_recurrence(L, lines, K)
    for ia, cac in enumerate(ca):
        for ib, cbc in enumerate(cb):
            tag = '%d_%d' % (ia, ib)
            sv = gen_hermite(la, lb, cac, cbc, K, lines, tag)
            lines.append(K + 'Yv[w][p][%d] = fmaf(f0v[p][%d], %s, Yv[w][p][%d]);'
                         % (ib, ia, sv, ib))
            if not diag:
                lines.append(K + 'Xv[w][p][%d] = fmaf(%s, h0v[p][%d], Xv[w][p][%d]);'
                             % (ia, sv, ib, ia))
    lines.append(J + '}')
    lines.append(J + '}')


def gen_class_dual(la, lb, diag):
    """Task body for two omegas at once (records staged in shared memory):
    the screen, headers, F loads and distances are shared, the integrals,
    accumulators and G_B updates are per omega slot (Gp[w * PTS + p],
    Xa[w * PTS * NCA + ...])."""
    nb = 2 * lb + 1
    nca = (la + 1) * (la + 2) // 2
    ncb = (lb + 1) * (lb + 2) // 2
    lines = []
    I = '    '
    J = I * 2
    lines.append('template<int PTS> struct CosxTask2<%d, %d, %s, PTS> {'
                 % (la, lb, 'true' if diag else 'false'))
    lines.append('static __device__ __forceinline__ void run(')
    lines.append('    float* const* Gp, const int ld, const int gb0,')
    lines.append('    const float4* __restrict__ rp, const int npp, const bool* ok,')
    lines.append('    const float* gxh, const float* gyh, const float* gzh,')
    lines.append('    const float* gxl, const float* gyl, const float* gzl,')
    lines.append('    const float4* __restrict__ stab, const float* f0,')
    lines.append('    const float* fb, float* Xa)')
    lines.append('{')
    lines.append(I + 'float f0v[PTS][%d], Yv[2][PTS][%d];' % (nca, ncb))
    if not diag:
        lines.append(I + 'float gbo[2][PTS][%d], h0v[PTS][%d], Xv[2][PTS][%d];'
                     % (nb, ncb, nca))
    lines.append(I + '#pragma unroll')
    lines.append(I + 'for (int p = 0; p < PTS; ++p) {')
    if not diag:
        lines.append(J + '#pragma unroll')
        lines.append(J + 'for (int w = 0; w < 2; ++w) {')
        lines.append('#if !WB_COSX_GB_RED')
        for nu in range(nb):
            lines.append(J + '    gbo[w][p][%d] = Gp[w * PTS + p][(long long)(gb0 + %d) * ld];'
                         % (nu, nu))
        lines.append('#endif')
        for c in range(nca):
            lines.append(J + '    Xv[w][p][%d] = Xa[(w * PTS + p) * %d + %d];' % (c, nca, c))
        lines.append(J + '}')
        for nu in range(nb):
            lines.append(J + 'const float fb%d = fb[p * %d + %d];' % (nu, nb, nu))
        gen_transform_in(lb, 'fb', 'h0_', J, lines)
        for c in range(ncb):
            lines.append(J + 'h0v[p][%d] = h0_%d;' % (c, c))
    for c in range(nca):
        lines.append(J + 'f0v[p][%d] = f0[p * %d + %d];' % (c, nca, c))
    for c in range(ncb):
        lines.append(J + 'Yv[0][p][%d] = 0.0f;' % c)
        lines.append(J + 'Yv[1][p][%d] = 0.0f;' % c)
    lines.append(I + '}')
    lines.append(I + '#pragma unroll 1')
    lines.append(I + 'for (int m = 0; m < npp; ++m) {')
    lines.append(J + 'const float4* __restrict__ q = rp + m * %d;' % rec_stride2(la, lb))
    lines.append(J + '{')
    gen_prim_body_dual(la, lb, diag, J + I, lines)
    lines.append(J + '}')
    lines.append(I + '}')
    lines.append(I + '#pragma unroll')
    lines.append(I + 'for (int w = 0; w < 2; ++w) {')
    lines.append(I + '#pragma unroll')
    lines.append(I + 'for (int p = 0; p < PTS; ++p) {')
    if diag:
        for c in range(ncb):
            lines.append(J + 'Xa[(w * PTS + p) * %d + %d] += Yv[w][p][%d];' % (nca, c, c))
    else:
        for c in range(ncb):
            lines.append(J + 'const float Y%d = Yv[w][p][%d];' % (c, c))
        gen_transform_out(lb, 'Y', 'gy', J, lines)
        lines.append(J + 'if (ok[p]) {')
        for nu in range(nb):
            lines.append('#if WB_COSX_GB_RED')
            lines.append(J + '    gb_add(Gp[w * PTS + p] + (long long)(gb0 + %d) * ld, gy%d);'
                         % (nu, nu))
            lines.append('#else')
            lines.append(J + '    Gp[w * PTS + p][(long long)(gb0 + %d) * ld] = gbo[w][p][%d] + gy%d;'
                         % (nu, nu, nu))
            lines.append('#endif')
        lines.append(J + '}')
        for c in range(nca):
            lines.append(J + 'Xa[(w * PTS + p) * %d + %d] = Xv[w][p][%d];' % (nca, c, c))
    lines.append(I + '}')
    lines.append(I + '}')
    lines.append('}')
    lines.append('};')
    return '\n'.join(lines)


def gen_class_dual_packed(la, lb, diag):
    """The PTS = 2 form of gen_class_dual: accumulators, F values and the
    lane's two grid points held as float2 pairs, the primitive-pair work
    on the packed FP32 instructions (bitwise the scalar form's results)."""
    nb = 2 * lb + 1
    nca = (la + 1) * (la + 2) // 2
    ncb = (lb + 1) * (lb + 2) // 2
    lines = []
    I = '    '
    J = I * 2
    lines.append('template<> struct CosxTask2<%d, %d, %s, 2> {'
                 % (la, lb, 'true' if diag else 'false'))
    lines.append('static __device__ __forceinline__ void run(')
    lines.append('    float* const* Gp, const int ld, const int gb0,')
    lines.append('    const float4* __restrict__ rp, const int npp, const bool* ok,')
    lines.append('    const float* gxh, const float* gyh, const float* gzh,')
    lines.append('    const float* gxl, const float* gyl, const float* gzl,')
    lines.append('    const float4* __restrict__ stab, const float* f0,')
    lines.append('    const float* fb, float* Xa)')
    lines.append('{')
    lines.append(I + 'constexpr int PTS = 2;')
    for ax in 'xyz':
        for hl in 'hl':
            lines.append(I + 'const float2 NG%s%s = make_float2(-g%s%s[0], -g%s%s[1]);'
                         % (ax.upper(), hl.upper(), ax, hl, ax, hl))
    lines.append(I + 'float2 f0p[%d], Yp[2][%d];' % (nca, ncb))
    for c in range(nca):
        lines.append(I + 'f0p[%d] = make_float2(f0[%d], f0[%d]);' % (c, c, nca + c))
    for c in range(ncb):
        lines.append(I + 'Yp[0][%d] = make_float2(0.0f, 0.0f);' % c)
        lines.append(I + 'Yp[1][%d] = make_float2(0.0f, 0.0f);' % c)
    if not diag:
        lines.append(I + 'float2 h0p[%d], Xp[2][%d];' % (ncb, nca))
        lines.append('#if !WB_COSX_GB_RED')
        lines.append(I + 'float gbo[2][PTS][%d];' % nb)
        lines.append(I + '#pragma unroll')
        lines.append(I + 'for (int w = 0; w < 2; ++w)')
        lines.append(I + '#pragma unroll')
        lines.append(I + 'for (int p = 0; p < PTS; ++p) {')
        for nu in range(nb):
            lines.append(J + 'gbo[w][p][%d] = Gp[w * PTS + p][(long long)(gb0 + %d) * ld];'
                         % (nu, nu))
        lines.append(I + '}')
        lines.append('#endif')
        lines.append(I + '#pragma unroll')
        lines.append(I + 'for (int w = 0; w < 2; ++w) {')
        for c in range(nca):
            lines.append(J + 'Xp[w][%d] = make_float2(Xa[(w * PTS) * %d + %d], '
                         'Xa[(w * PTS + 1) * %d + %d]);' % (c, nca, c, nca, c))
        lines.append(I + '}')
        for p in range(2):
            for nu in range(nb):
                lines.append(I + 'const float fb%d_%d = fb[%d];' % (p, nu, p * nb + nu))
            gen_transform_in(lb, 'fb%d_' % p, 'h%d_' % p, I, lines)
        for c in range(ncb):
            lines.append(I + 'h0p[%d] = make_float2(h0_%d, h1_%d);' % (c, c, c))
    lines.append(I + '#pragma unroll 1')
    lines.append(I + 'for (int m = 0; m < npp; ++m) {')
    lines.append(J + 'const float4* __restrict__ q = rp + m * %d;' % rec_stride2(la, lb))
    lines.append(J + '{')
    gen_prim_body_dual(la, lb, diag, J + I, lines, packed=True)
    lines.append(J + '}')
    lines.append(I + '}')
    lines.append(I + '#pragma unroll')
    lines.append(I + 'for (int w = 0; w < 2; ++w) {')
    for p in range(2):
        h = 'xy'[p]
        lines.append(I + '{')
        if diag:
            for c in range(ncb):
                lines.append(J + 'Xa[(w * PTS + %d) * %d + %d] += Yp[w][%d].%s;'
                             % (p, nca, c, c, h))
        else:
            for c in range(ncb):
                lines.append(J + 'const float Y%d = Yp[w][%d].%s;' % (c, c, h))
            gen_transform_out(lb, 'Y', 'gy', J, lines)
            lines.append(J + 'if (ok[%d]) {' % p)
            for nu in range(nb):
                lines.append('#if WB_COSX_GB_RED')
                lines.append(J + '    gb_add(Gp[w * PTS + %d] + (long long)(gb0 + %d) * ld, gy%d);'
                             % (p, nu, nu))
                lines.append('#else')
                lines.append(J + '    Gp[w * PTS + %d][(long long)(gb0 + %d) * ld] = gbo[w][%d][%d] + gy%d;'
                             % (p, nu, p, nu, nu))
                lines.append('#endif')
            lines.append(J + '}')
            for c in range(nca):
                lines.append(J + 'Xa[(w * PTS + %d) * %d + %d] = Xp[w][%d].%s;'
                             % (p, nca, c, c, h))
        lines.append(I + '}')
    lines.append(I + '}')
    lines.append('}')
    lines.append('};')
    return '\n'.join(lines)


def source():
    out = ['// Generated by csrc/gen_cosx.py -- do not edit by hand.',
           '// One straight-line task body per shell-pair class (la >= lb),',
           '// its primitive-pair record and loader, plus the per-run begin',
           '// (F_A -> Cartesian f0) and end (G_A = c2s^T X) of each bra',
           '// angular momentum.',
           '#pragma once', '']
    for la in range(LMAX + 1):
        out.append(gen_begin(la))
        out.append('')
        out.append(gen_end(la))
        out.append('')
    for (la, lb) in classes():
        out.append(gen_rec(la, lb))
        out.append('')
    for (la, lb) in classes():
        for far in (False, True):
            for stage in (False, True):
                out.append(gen_class(la, lb, False, far, stage))
                out.append('')
                if la == lb:
                    out.append(gen_class(la, lb, True, far, stage))
                    out.append('')
        out.append(gen_class_dual(la, lb, False))
        out.append('')
        if la == lb:
            out.append(gen_class_dual(la, lb, True))
            out.append('')
        if la + lb <= 3:
            out.append('#if WB_COSX_F32X2')
            out.append(gen_class_dual_packed(la, lb, False))
            if la == lb:
                out.append('')
                out.append(gen_class_dual_packed(la, lb, True))
            out.append('#endif')
            out.append('')
    # E strides table for the host
    out.append('#define WB_E_STRIDES {%s}' % ', '.join(
        str(e_stride(la, lb)) for (la, lb) in classes()))
    out.append('')
    return '\n'.join(out)


def layout_source():
    """Host-visible constants of the packed primitive-pair records."""
    cl = classes()
    return '\n'.join([
        '// Generated by csrc/gen_cosx.py -- do not edit by hand.',
        '// Packed primitive-pair record of each class (class order):',
        '// float4 count = 2 (P hi, P lo) + n_om (omega record) + n_e (E).',
        '#pragma once', '',
        'namespace wb {',
        'constexpr int kRecNom[10] = {%s};' % ', '.join(str(n_om(a, b)) for a, b in cl),
        'constexpr int kRecNe[10] = {%s};' % ', '.join(str(e_stride(a, b) // 4) for a, b in cl),
        'constexpr int kRecStride[10] = {%s};' % ', '.join(str(rec_stride(a, b)) for a, b in cl),
        '// dual-omega record: 2 + 2 n_om + n_e',
        'constexpr int kRecStride2[10] = {%s};' % ', '.join(str(rec_stride2(a, b)) for a, b in cl),
        '}  // namespace wb', ''])


def _hartree_ridx(L, t, u, v):
    """Packed index of R_tuv (t + u + v <= L): v-major, then u, then t."""
    k = 0
    for vv in range(v):
        for uu in range(L - vv + 1):
            k += L - vv - uu + 1
    for uu in range(u):
        k += L - v - uu + 1
    return k + t


def hartree_source():
    """Straight-line Hermite Coulomb sums of the Hartree-potential kernel
    (csrc/scf_kernels.cu): for L = 0..6,

        hermite_dot_L(r0, x, y, z, dh) = sum_{t+u+v<=L} dh[idx(t,u,v)] R_tuv

    with R^(n)_000 = r0[n] and the McMurchie-Davidson recurrence
    R^(n)_{t+1,u,v} = t R^(n+1)_{t-1,u,v} + x R^(n+1)_{t,u,v} (u, v the same
    with y, z), written level by level as named values (no in-place
    array), so the compiler sees plain register code."""
    out = ['// Generated by csrc/gen_cosx.py (hartree_source); do not edit.',
           '#pragma once', '', 'namespace wb {', 'namespace scf {', '',
           '// four consecutive Hermite-density entries (a 16-byte aligned',
           '// block: float4, or two double2)',
           'template<typename Real> struct Hq4 { Real x, y, z, w; };',
           '__device__ __forceinline__ Hq4<float> ld_hq4(const float* p) {',
           '    const float4 v = __ldg(reinterpret_cast<const float4*>(p));',
           '    return {v.x, v.y, v.z, v.w};',
           '}',
           '__device__ __forceinline__ Hq4<double> ld_hq4(const double* p) {',
           '    const double2 a = __ldg(reinterpret_cast<const double2*>(p));',
           '    const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);',
           '    return {a.x, a.y, b.x, b.y};',
           '}',
           '']
    for L in range(7):
        out.append('template<typename Real>')
        out.append('__device__ __forceinline__ Real hermite_dot_%d(const Real* r0, '
                   'const Real x, const Real y, const Real z, const Real* dh) {' % L)
        names = {}

        def nm(n, t, u, v):
            return 'r%d_%d_%d_%d' % (n, t, u, v)
        for n in range(L, -1, -1):
            m = L - n
            for v in range(m + 1):
                for u in range(m + 1 - v):
                    for t in range(m + 1 - u - v):
                        if t == u == v == 0:
                            expr = 'r0[%d]' % n
                        elif t > 0:
                            a = nm(n + 1, t - 1, u, v)
                            expr = 'x * %s' % a
                            if t >= 2:
                                expr = 'Real(%d) * %s + %s' % (t - 1, nm(n + 1, t - 2, u, v), expr)
                        elif u > 0:
                            a = nm(n + 1, 0, u - 1, v)
                            expr = 'y * %s' % a
                            if u >= 2:
                                expr = 'Real(%d) * %s + %s' % (u - 1, nm(n + 1, 0, u - 2, v), expr)
                        else:
                            a = nm(n + 1, 0, 0, v - 1)
                            expr = 'z * %s' % a
                            if v >= 2:
                                expr = 'Real(%d) * %s + %s' % (v - 1, nm(n + 1, 0, 0, v - 2), expr)
                        out.append('    const Real %s = %s;' % (nm(n, t, u, v), expr))
        terms = []
        for v in range(L + 1):
            for u in range(L + 1 - v):
                for t in range(L + 1 - u - v):
                    terms.append((_hartree_ridx(L, t, u, v), nm(0, t, u, v)))
        terms.sort()
        # dh is read four entries at a time (its block is padded to a
        # multiple of 4); the sum keeps the entry order
        for g in range((len(terms) + 3) // 4):
            out.append('    const Hq4<Real> d%d = ld_hq4(dh + %d);' % (g, 4 * g))
        out.append('    Real s = Real(0);')
        for q, name in terms:
            out.append('    s += d%d.%s * %s;' % (q // 4, 'xyzw'[q % 4], name))
        out.append('    return s;')
        out.append('}')
        out.append('')
    out += ['}  // namespace scf', '}  // namespace wb', '']
    return '\n'.join(out)


def _write_if_changed(path, src):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    old = None
    if os.path.exists(path):
        with open(path) as fh:
            old = fh.read()
    if old != src:
        with open(path, 'w') as fh:
            fh.write(src)


def write(path=None):
    if path is None:
        path = os.path.join(HERE, 'generated', 'cosx_classes.cuh')
    _write_if_changed(path, source())
    _write_if_changed(os.path.join(os.path.dirname(path), 'cosx_layout.h'),
                      layout_source())
    _write_if_changed(os.path.join(os.path.dirname(path), 'hartree_r.cuh'),
                      hartree_source())
    return path


if __name__ == '__main__':
    print(write())
