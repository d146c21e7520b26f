"""Constrained transport restated in NumPy from the Fortran, against the
oracle's C++ on the same state: the face velocities of CC(1)
(3DMHD-CfCA/MCF3DSGincfca3.f90:2126-2134), the edge densities of CC(2)
(:2140-2157), CCT (:2186-2445) — VLIMIT's face-array slopes (:1777-1797)
with their T < 3 switch to minmod, the four corner candidates of the two
characteristic pairs, the upwind weights with the 1e13 boost where both
pairs agree, the weighted characteristics and the EMF — and the face-field
update of CC(3) (:2159-2169).  Each edge direction is worked in its own
frame (a, b, c) = (x, y, z), (y, z, x), (z, x, y), like the reference's
iwx / iwy / iwz branches.  The arithmetic is the reference's in its order
(the z-x edge density sums its four cells in another order than the other
two), so the two agree bit for bit.  The oracle supplies only the ghost
layers CC(1) exchanges."""
import numpy as np

from code_tohoku_gb300 import problems
from oracle.pyoracle import Oracle3D

EPS = 1e-10


def fmin2(a, b):
    return np.where(b < a, b, a)


def face_slope(q, u1, u5, dxp, kb, lo, hi):
    """VLIMIT for a face array along axis 0 at padded indices lo..hi (every
    index of the two other axes), with the temperature of the cell of the
    same index; dxp the padded widths along that axis."""
    qp, q0, qm = q[lo + 1:hi + 2], q[lo:hi + 1], q[lo - 1:hi]
    d0 = dxp[lo:hi + 1][:, None, None]
    dm = dxp[lo - 1:hi][:, None, None]
    dp = dxp[lo + 1:hi + 2][:, None, None]
    delp = qp - q0
    delm = q0 - qm
    x = (2.0 * delp * delm + EPS) / (delp * delp + delm * delm + EPS)
    flmt = np.where(x > 0.0, x, 0.0)
    g = flmt * (qp - qm) / (d0 + 0.5 * dm + 0.5 * dp)
    T = 1.27 * u5[lo:hi + 1] / (kb * u1[lo:hi + 1])
    delp = 2.0 * delp / (d0 + dp)
    delm = 2.0 * delm / (d0 + dm)
    gmm = (0.5 + np.copysign(0.5, delp * delm)) * np.copysign(1.0, delp) * fmin2(np.abs(delp), np.abs(delm))
    return g * (0.5 - np.copysign(0.5, T - 3.0)) + gmm * (0.5 + np.copysign(0.5, T - 3.0))


def local(A, e):
    """Array [z, y, x] in the frame of edge direction e: axes (a, b, c)."""
    da, db, dc = e, (e + 1) % 3, (e + 2) % 3
    return np.transpose(A, (2 - da, 2 - db, 2 - dc))


def emf_edge(e, U, Vfc, dx, n, kb, facdep, dt, stats=None):
    """EMF along edge direction e at a = 1..Na+1, b = 1..Nb+1, c = 1..Nc, in
    the local frame (padded indices 2..Na+2, 2..Nb+2, 2..Nc+1)."""
    da, db, dc = e, (e + 1) % 3, (e + 2) % 3
    Na, Nb, Nc = n[da], n[db], n[dc]
    r, p = local(U[0], e), local(U[4], e)
    Vx, Vy = local(Vfc[da], e), local(Vfc[db], e)
    Bx, By = local(U[5 + da], e), local(U[5 + db], e)
    dxe, dye = dx[da], dx[db]
    A = slice(2, Na + 3)
    B = slice(2, Nb + 3)
    C = slice(2, Nc + 2)
    # dnc of CC(2): four cells around the edge; the z-x edge adds them in
    # the reference's own order
    if e == 2:
        dnc = 0.25 * (r[2:Na + 3, 2:Nb + 3] + r[2:Na + 3, 1:Nb + 2] + r[1:Na + 2, 2:Nb + 3] + r[1:Na + 2, 1:Nb + 2])
    else:
        dnc = 0.25 * (r[2:Na + 3, 2:Nb + 3] + r[1:Na + 2, 2:Nb + 3] + r[2:Na + 3, 1:Nb + 2] + r[1:Na + 2, 1:Nb + 2])
    dnc = dnc[:, :, C]
    with np.errstate(all="ignore"):
        # slopes along a at a = 0..Na+1 (padded 1..Na+2), along b at b = 0..Nb+1
        dQ2 = np.zeros_like(Vy)
        dQ4 = np.zeros_like(Vy)
        dQ2[1:Na + 3] = face_slope(Vy, r, p, dxe, kb, 1, Na + 2)
        dQ4[1:Na + 3] = face_slope(By, r, p, dxe, kb, 1, Na + 2)
        sw = lambda q: np.swapaxes(q, 0, 1)
        dQ1 = np.zeros_like(Vx)
        dQ3 = np.zeros_like(Vx)
        sw(dQ1)[1:Nb + 3] = face_slope(sw(Vx), sw(r), sw(p), dye, kb, 1, Nb + 2)
        sw(dQ3)[1:Nb + 3] = face_slope(sw(Bx), sw(r), sw(p), dye, kb, 1, Nb + 2)
    facm = facdep * 0.5
    dsqinv = 1.0 / np.sqrt(dnc)
    at = lambda q, sa, sb: q[2 + sa:Na + 3 + sa, 2 + sb:Nb + 3 + sb, C]

    def one(sa1, sb1, sa2, sb2, dy, dxw, S1, S2):
        # the field at a-face offset (0, sb1) and the b-face offset (sa2, 0)
        a1p = at(Vx, sa1, sb1) + at(Bx, sa1, sb1) * dsqinv
        da1p = (at(dQ1, sa1, sb1) + at(dQ3, sa1, sb1) * dsqinv) * facm
        a1m = at(Vx, sa1, sb1) - at(Bx, sa1, sb1) * dsqinv
        da1m = (at(dQ1, sa1, sb1) - at(dQ3, sa1, sb1) * dsqinv) * facm
        a2m = at(Vy, sa2, sb2) - at(By, sa2, sb2) * dsqinv
        da2m = (at(dQ2, sa2, sb2) - at(dQ4, sa2, sb2) * dsqinv) * facm
        a2p = at(Vy, sa2, sb2) + at(By, sa2, sb2) * dsqinv
        da2p = (at(dQ2, sa2, sb2) + at(dQ4, sa2, sb2) * dsqinv) * facm
        c1p = (a1p + da1p * dy * S1 - da1p * (a2m + da2m * dxw * S2) * dt) / (1.0 - da1p * da2m * dt * dt)
        c2m = (a2m + da2m * dxw * S2 - da2m * (a1p + da1p * dy * S1) * dt) / (1.0 - da1p * da2m * dt * dt)
        c1m = (a1m + da1m * dy * S1 - da1m * (a2p + da2p * dxw * S2) * dt) / (1.0 - da1m * da2p * dt * dt)
        c2p = (a2p + da2p * dxw * S2 - da2p * (a1m + da1m * dy * S1) * dt) / (1.0 - da1m * da2p * dt * dt)
        return c1p, c2m, c1m, c2p

    dym = dye[1:Nb + 2][None, :, None]   # dye(j-1), j = 1..Nb+1
    dy0 = dye[2:Nb + 3][None, :, None]
    dxm = dxe[1:Na + 2][:, None, None]
    dx0 = dxe[2:Na + 3][:, None, None]
    LL = one(0, -1, -1, 0, dym, dxm, 1.0, 1.0)     # C1 > 0, C2 > 0
    RL = one(0, 0, -1, 0, dy0, dxm, -1.0, 1.0)     # C1 > 0, C2 < 0
    LR = one(0, -1, 0, 0, dym, dx0, 1.0, -1.0)     # C1 < 0, C2 > 0
    RR = one(0, 0, 0, 0, dy0, dx0, -1.0, -1.0)     # C1 < 0, C2 < 0
    cand = (LL, RL, LR, RR)
    s1 = (1, 1, -1, -1)    # the sign of C1 each corner wants
    s2 = (1, -1, 1, -1)    # the sign of C2
    want = lambda v, s: (v > 0.0) if s > 0 else (v < 0.0)
    ifw1 = [want(c[0], s1[m]) & want(c[1], s2[m]) for m, c in enumerate(cand)]   # (C1p, C2m)
    ifw2 = [want(c[2], s1[m]) & want(c[3], s2[m]) for m, c in enumerate(cand)]   # (C1m, C2p)
    W1, W2 = [], []
    for m in range(4):
        boost = np.trunc(0.51 * ifw1[m] + 0.51 * ifw2[m])
        W1.append(ifw1[m] + (1.e13 - 1.0) * boost)
        W2.append(ifw2[m] + (1.e13 - 1.0) * boost)
    any1 = (ifw1[0].astype(int) + ifw1[1] + ifw1[2] + ifw1[3]) != 0
    any2 = (ifw2[0].astype(int) + ifw2[1] + ifw2[2] + ifw2[3]) != 0

    def weighted(W, x, y):
        # sum_m W_m |y_m| x_m / sum_m W_m |y_m|, left to right
        num = W[0] * np.abs(y[0]) * x[0] + W[1] * np.abs(y[1]) * x[1] + W[2] * np.abs(y[2]) * x[2] \
            + W[3] * np.abs(y[3]) * x[3]
        den = W[0] * np.abs(y[0]) + W[1] * np.abs(y[1]) + W[2] * np.abs(y[2]) + W[3] * np.abs(y[3])
        return num, den

    with np.errstate(all="ignore"):
        n1, d1 = weighted(W1, [c[0] for c in cand], [c[1] for c in cand])
        C1p = np.where(any1, n1 / d1, 0.0)
        n1, d1 = weighted(W1, [c[1] for c in cand], [c[0] for c in cand])
        C2m = np.where(any1, n1 / d1, 0.0)
        n2, d2 = weighted(W2, [c[2] for c in cand], [c[3] for c in cand])
        C1m = np.where(any2, n2 / d2, 0.0)
        n2, d2 = weighted(W2, [c[3] for c in cand], [c[2] for c in cand])
        C2p = np.where(any2, n2 / d2, 0.0)
    v1a, v2a, B1a, B2a = C1p + C1m, C2p + C2m, C1p - C1m, C2p - C2m
    if stats is not None:
        stats["boost"] = stats.get("boost", 0) + int(sum(np.count_nonzero(ifw1[m] & ifw2[m]) for m in range(4)))
        stats["none"] = stats.get("none", 0) + int(np.count_nonzero(~any1 | ~any2))
        stats["mixed"] = stats.get("mixed", 0) + int(np.count_nonzero(
            (np.add.reduce([w.astype(int) for w in ifw1]) > 1)))
        T = 1.27 * p[2:-2, 2:-2, 2:-2] / (kb * r[2:-2, 2:-2, 2:-2])
        stats["cold"] = stats.get("cold", 0) + int(np.count_nonzero(T < 3.0))
        stats["warm"] = stats.get("warm", 0) + int(np.count_nonzero(T > 3.0))
    return 0.25 * (v1a * B2a - v2a * B1a) * np.sqrt(dnc)


def face_velocities(U, dx, n):
    """CC(1)'s Vfc on its faces: x faces i = 1..Nx+1 (j, k interior), etc.,
    as [z, y, x] slices of the padded arrays."""
    nx, ny, nz = n
    out = []
    for d in range(3):
        v = local(U[1 + d], d)        # axis 0 along d
        w = dx[d]
        lo, hi = 2, n[d] + 2          # padded face indices 2..N+2
        dm = w[lo - 1:hi][:, None, None]
        d0 = w[lo:hi + 1][:, None, None]
        f = (dm * v[lo:hi + 1] + d0 * v[lo - 1:hi]) / (dm + d0)
        # interior of the two transverse directions
        out.append(f[:, 2:n[(d + 1) % 3] + 2, 2:n[(d + 2) % 3] + 2])
    return out


def make_state(n, seed):
    st = problems.colliding_flows(n)
    rng = np.random.default_rng(seed)
    for d in range(3):   # cell widths vary, so every index of dx counts
        w = st.dx if d == 0 else (st.dy if d == 1 else st.dz)
        w *= rng.uniform(0.7, 1.3, w.shape)
    st.U[0] *= rng.uniform(0.5, 1.5, st.U[0].shape)
    for q in (1, 2, 3):
        st.U[q] += rng.normal(0.0, 8.0, st.U[q].shape)
    for q in (5, 6, 7):
        st.U[q] += rng.normal(0.0, 6.0, st.U[q].shape)
    # T in 1e3 K on both sides of the 3 (3000 K) switch of VLIMIT
    T = rng.uniform(1.0, 6.0, st.U[0].shape)
    st.U[4][...] = T * problems.KB * st.U[0] / 1.27
    return st


def test_ct_matches_an_independent_restatement():
    st = make_state(14, 5)
    p = st.params
    n = (p.nx, p.ny, p.nz)
    dx = (st.dx, st.dy, st.dz)
    dt = 0.02
    o = Oracle3D(p)
    o.upload(st)
    U, Vfc, EMF, Bnew = o.ct_probe(dt)

    # face velocities
    vf = face_velocities(U, dx, n)
    for d in range(3):
        got = local(Vfc[d], d)[2:n[d] + 3, 2:n[(d + 1) % 3] + 2, 2:n[(d + 2) % 3] + 2]
        assert np.array_equal(got, vf[d]), d

    # EMF of each edge direction, in its own frame
    ez = (2, 0, 1)   # EMF slot of Ez (e = 0), Ex (e = 1), Ey (e = 2)
    stats = {}
    mine = []
    for e in range(3):
        da, db, dc = e, (e + 1) % 3, (e + 2) % 3
        E = emf_edge(e, U, Vfc, dx, n, p.kb, p.facdep, dt, stats)
        got = local(EMF[ez[e]], e)[2:n[da] + 3, 2:n[db] + 3, 2:n[dc] + 2]
        assert np.array_equal(got, E), e
        full = np.zeros_like(U[0])
        local(full, e)[2:n[da] + 3, 2:n[db] + 3, 2:n[dc] + 2] = E
        mine.append(full)
    # every branch of the upwinding and of the slope switch was taken
    assert stats["boost"] > 0 and stats["none"] > 0 and stats["mixed"] > 0, stats
    assert stats["cold"] > 0 and stats["warm"] > 0, stats

    # CC(3): the face fields from the EMF's circulation
    Ex, Ey, Ez = mine[1], mine[2], mine[0]
    nx, ny, nz = n
    dxp, dyp, dzp = (w[:, None, None] for w in dx)
    K, J, I = slice(2, nz + 2), slice(2, ny + 2), slice(2, nx + 2)
    dyj, dzk, dxi = st.dy[J][None, :, None], st.dz[K][:, None, None], st.dx[I][None, None, :]
    I1, J1, K1 = slice(2, nx + 3), slice(2, ny + 3), slice(2, nz + 3)
    sh = lambda s: slice(s.start + 1, s.stop + 1)
    b1 = U[5][K, J, I1] + dt / dyj * (Ez[K, sh(J), I1] - Ez[K, J, I1]) \
        - dt / dzk * (Ey[sh(K), J, I1] - Ey[K, J, I1])
    b2 = U[6][K, J1, I] + dt / dzk * (Ex[sh(K), J1, I] - Ex[K, J1, I]) \
        - dt / dxi * (Ez[K, J1, sh(I)] - Ez[K, J1, I])
    b3 = U[7][K1, J, I] + dt / dxi * (Ey[K1, J, sh(I)] - Ey[K1, J, I]) \
        - dt / dyj * (Ex[K1, sh(J), I] - Ex[K1, J, I])
    assert np.array_equal(Bnew[0][K, J, I1], b1)
    assert np.array_equal(Bnew[1][K, J1, I], b2)
    assert np.array_equal(Bnew[2][K1, J, I], b3)
    assert np.any(Bnew[0][K, J, I1] != U[5][K, J, I1])
