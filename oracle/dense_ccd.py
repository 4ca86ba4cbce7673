"""Independent dense-tensor CCD in numpy, used to validate the oracle (test infrastructure).

Everything here is written from the textbook spin-orbital CCD equations, not from
the reference's channel factorisation:

  0 = <ab|V|ij> + P(ab) f_bc t^ac_ij - P(ij) f_kj t^ab_ik
      + 1/2 <ab|V|cd> t^cd_ij + 1/2 <kl|V|ij> t^ab_kl + P(ij)P(ab) <kb|V|cj> t^ac_ik
      + 1/4 <kl|V|cd> t^cd_ij t^ab_kl + 1/2 P(ij)P(ab) <kl|V|cd> t^ac_ik t^bd_jl
      - 1/2 P(ab) <kl|V|cd> t^ac_ij t^bd_kl - 1/2 P(ij) <kl|V|cd> t^ab_ik t^cd_jl

with the amplitude stored as T(ab,ij) and <ab|V|ij> taken as conj(<ij|V|ab>) the
way the reference builds its right-hand side (ccm_t2_eqn.f90:106-138).  The
potential is evaluated here vectorised over all four orbitals from the orbit table,
independently of the oracle's per-element routine, so the check also covers the
Minnesota formula and the antisymmetrisation.  Sizes: nmax=1 lattices only.
"""
from __future__ import annotations

import numpy as np

PI = 3.14159265358979
F32 = lambda x: float(np.float32(x))  # noqa: E731  default-real literal of the reference


def minnesota_dense(orb: dict, volume: float, f32_literals: bool = True) -> np.ndarray:
    """Bare (non-antisymmetrised) Minnesota v(p,q,r,s) over all orbitals."""
    kx, ky, kz = orb["kx"], orb["ky"], orb["kz"]
    n = len(kx)
    nx, ny, nz, sz, tz = orb["nx"], orb["ny"], orb["nz"], orb["sz"], orb["tz"]
    k = np.stack([kx, ky, kz], axis=1)
    P, Q, R, S = np.ix_(np.arange(n), np.arange(n), np.arange(n), np.arange(n))
    cons = ((nx[P] + nx[Q]) == (nx[R] + nx[S])) & ((ny[P] + ny[Q]) == (ny[R] + ny[S])) & \
        ((nz[P] + nz[Q]) == (nz[R] + nz[S])) & ((tz[P] + tz[Q]) == (tz[R] + tz[S]))
    prel = 0.5 * (k[:, None, :] - k[None, :, :])  # (p,q,3)
    q = prel[:, :, None, None, :] - prel[None, None, :, :, :]
    q2 = (q[..., 0] * q[..., 0] + q[..., 1] * q[..., 1]) + q[..., 2] * q[..., 2]
    c = F32 if f32_literals else float
    v0r, v0t, v0s = c(200.0), c(178.0), c(91.85)
    kr, kt, ks = c(1.487), c(0.639), c(0.465)
    pi15 = PI ** 1.5
    vr = v0r * pi15 * np.exp(-q2 / (4.0 * kr)) / kr ** 1.5
    vt = -v0t * pi15 * np.exp(-q2 / (4.0 * kt)) / kt ** 1.5
    vs = -v0s * pi15 * np.exp(-q2 / (4.0 * ks)) / ks ** 1.5

    def pdot(m1, m2, m3, m4):
        nf = (m1 == m3) & (m2 == m4)
        ex = (m1 == m4) & (m2 == m3) & (m1 != m2)
        return np.where(nf, (m1 * m2).astype(float), np.where(ex, 2.0, 0.0))

    m1, m2, m3, m4 = sz[P], sz[Q], sz[R], sz[S]
    t1, t2, t3, t4 = tz[P], tz[Q], tz[R], tz[S]
    dm = ((m1 == m3) & (m2 == m4)).astype(float)
    dt = ((t1 == t3) & (t2 == t4)).astype(float)
    tt = pdot(t1, t2, t3, t4)
    ss = pdot(m1, m2, m3, m4)
    vr = vr * (3.0 * dm * dt - tt * dm - ss * dt - tt * ss) / 8.0
    vs = vs * (3.0 * dm * dt + tt * dm - 3.0 * ss * dt - tt * ss) / 16.0
    vt = vt * (3.0 * dm * dt - 3.0 * tt * dm + ss * dt - tt * ss) / 16.0
    v = ((vs + vr) + vt) / volume
    return np.where(cons, v, 0.0).astype(np.complex128)


class DenseCCD:
    def __init__(self, orb: dict, A: int, vbare: np.ndarray):
        self.A = A
        n = len(orb["e"])
        self.n = n
        V = vbare - vbare.transpose(0, 1, 3, 2)  # <pq|V|rs>_A
        self.V = V
        h = slice(0, A)
        p = slice(A, n)
        # Fock: t + sum_h <h p|V|h q>  (momentum diagonal by construction)
        f = np.diag(np.asarray(orb["e"], dtype=np.complex128))
        f = f + np.einsum("hphq->pq", V[h, :, h, :])
        self.f = f
        self.e0 = np.sum(orb["e"][:A]) + 0.5 * np.einsum("ijij->", V[h, h, h, h])
        self.fhh = f[h, h]
        self.fpp = f[p, p]
        self.v_ijab = V[h, h, p, p]
        self.v_abij = np.conj(self.v_ijab).transpose(2, 3, 0, 1)  # conj(<ij|V|ab>)
        self.v_abcd = V[p, p, p, p]
        self.v_klij = V[h, h, h, h]
        self.v_kbcj = V[h, p, p, h]
        self.v_klcd = V[h, h, p, p]
        fo = np.real(np.diag(self.fhh))
        fv = np.real(np.diag(self.fpp))
        self.D0 = fo[None, None, :, None] + fo[None, None, None, :] - fv[:, None, None, None] - fv[None, :, None, None]

    def mp2(self) -> np.ndarray:
        D = self.D0
        with np.errstate(divide="ignore", invalid="ignore"):
            t = np.where(np.abs(D) == 0.0, 0.0, self.v_abij / D)
        return t.astype(np.complex128)

    def energy(self, t: np.ndarray) -> complex:
        # 1/4 sum T(ab,ij) V(ij,ab)
        return 0.25 * np.einsum("abij,ijab->", t, self.v_ijab)

    def residual(self, t: np.ndarray) -> np.ndarray:
        """Full textbook right-hand side including the diagonal Fock terms."""
        V = self.v_klcd
        r = self.v_abij.copy()
        x = np.einsum("bc,acij->abij", self.fpp, t)
        r += x - x.transpose(1, 0, 2, 3)
        x = -np.einsum("kj,abik->abij", self.fhh, t)
        r += x - x.transpose(0, 1, 3, 2)
        r += 0.5 * np.einsum("abcd,cdij->abij", self.v_abcd, t)
        r += 0.5 * np.einsum("klij,abkl->abij", self.v_klij, t)
        x = np.einsum("kbcj,acik->abij", self.v_kbcj, t)
        r += x - x.transpose(1, 0, 2, 3) - x.transpose(0, 1, 3, 2) + x.transpose(1, 0, 3, 2)
        r += 0.25 * np.einsum("klcd,cdij,abkl->abij", V, t, t, optimize=True)
        x = 0.5 * np.einsum("klcd,acik,bdjl->abij", V, t, t, optimize=True)
        r += x - x.transpose(1, 0, 2, 3) - x.transpose(0, 1, 3, 2) + x.transpose(1, 0, 3, 2)
        x = -0.5 * np.einsum("klcd,acij,bdkl->abij", V, t, t, optimize=True)
        r += x - x.transpose(1, 0, 2, 3)
        x = -0.5 * np.einsum("klcd,abik,cdjl->abij", V, t, t, optimize=True)
        r += x - x.transpose(0, 1, 3, 2)
        return r

    def solve(self, tol: float = 1e-11, max_iter: int = 200, diis: int = 8):
        t = self.mp2()
        D = self.D0
        hist_t, hist_e = [], []
        for it in range(max_iter):
            r = self.residual(t)
            rn = np.linalg.norm(r)
            if rn < tol:
                return t, it, rn
            with np.errstate(divide="ignore", invalid="ignore"):
                step = np.where(np.abs(D) == 0.0, 0.0, r / D)
            tj = t + step
            hist_t.append(tj)
            hist_e.append(step)
            if len(hist_t) > diis:
                hist_t.pop(0)
                hist_e.pop(0)
            m = len(hist_t)
            if m >= 2:
                B = np.zeros((m + 1, m + 1))
                for i in range(m):
                    for j in range(m):
                        B[i, j] = np.real(np.vdot(hist_e[i], hist_e[j]))
                B[:m, m] = -1.0
                B[m, :m] = -1.0
                rhs = np.zeros(m + 1)
                rhs[m] = -1.0
                c = np.linalg.solve(B, rhs)
                t = sum(c[i] * hist_t[i] for i in range(m))
            else:
                t = tj
        return t, max_iter, rn


def triples_dense(d: DenseCCD, t: np.ndarray) -> complex:
    """[T] energy from textbook connected triples, real interaction assumed:
    W = P(i/jk)P(a/bc)[sum_e T(ae,jk) <ei|V|bc> - sum_m T(bc,im) <ma|V|jk>],
    E = sum_{i<j<k, a<b<c} |W|^2 / (f_i+f_j+f_k-f_a-f_b-f_c)."""
    A = d.A
    n = d.n
    V = d.V
    h = np.arange(A)
    p = np.arange(A, n)
    v_eibc = V[np.ix_(p, h, p, p)]  # (e,i,b,c)
    v_majk = V[np.ix_(h, p, h, h)]  # (m,a,j,k)
    fo = np.real(np.diag(d.fhh))
    fv = np.real(np.diag(d.fpp))
    Dv = fv[:, None, None] + fv[None, :, None] + fv[None, None, :]
    a_, b_, c_ = np.meshgrid(np.arange(len(p)), np.arange(len(p)), np.arange(len(p)), indexing="ij")
    mask = (a_ < b_) & (b_ < c_)

    def X(i, j, k):
        return np.einsum("ae,ebc->abc", t[:, :, j, k], v_eibc[:, i]) - \
            np.einsum("bcm,ma->abc", t[:, :, i, :], v_majk[:, :, j, k])

    def Pa(g):
        return g - g.transpose(1, 0, 2) - g.transpose(2, 1, 0)

    e = 0.0 + 0.0j
    for i in range(A):
        for j in range(i + 1, A):
            for k in range(j + 1, A):
                w = Pa(X(i, j, k)) - Pa(X(j, i, k)) - Pa(X(k, j, i))
                D = fo[i] + fo[j] + fo[k] - Dv
                e += np.sum(np.where(mask, np.conj(w) * w / D, 0.0))
    return e
