"""Oracle: streamed NumPy float64 restatement of ``hqc/pbc/solver.py`` (Gamma).

Test infrastructure only (see ``oracle/__init__.py``).  Every function cites
the reference lines it restates.  Grid points are ordered (x, y, z) in C order
with x_i = i L / n; sums over the grid and over the (odd) frequency cube are
independent of that ordering, so results equal the reference's up to rounding.
"""
import numpy as np

from .basis import Basis
from . import xc as xcmod

RY = 2.0
MADELUNG_SC = 0.22578495  # hqc/pbc/solver.py:404 (4*pi*0.22578495 = 2.8372975)


class Setup:
    """Factory-time tables, ``hqc/pbc/solver.py:14-231``."""

    def __init__(self, n, L, rs, basis, rcut=24.0, grid_length=0.12, n_grid=None):
        self.n = n
        self.rs = rs
        self.L = L * rs  # Bohr (solver.py:154)
        self.Omega = self.L ** 3
        self.basis = Basis(basis) if isinstance(basis, str) else basis
        self.nao_atom = self.basis.nao
        self.nao = n * self.nao_atom
        # odd grid (solver.py:159)
        self.ng = n_grid if n_grid is not None else int(round(self.L / grid_length / 2)) * 2 + 1
        self.N = self.ng ** 3
        self.dV = self.Omega / self.N
        self.x1d = np.arange(self.ng) * self.L / self.ng  # Rmesh_1d (solver.py:190)
        # GTO 1D lattice: tmax = 24 // L, the grid lattice always uses rcut 24
        # because make_pbc_gto is called without rcut (solver.py:211, gto.py:48)
        tmax1 = 24.0 // self.L
        self.lat1d = np.arange(-tmax1, tmax1 + 1) * self.L
        # S/T lattice sphere (solver.py:162-176)
        tmax = rcut // self.L
        nt = np.arange(-tmax, tmax + 1)
        T = np.array(np.meshgrid(nt, nt, nt)).reshape(3, -1).T * self.L
        self.lattice = T[(T ** 2).sum(1) <= rcut ** 2]
        # frequencies in numpy FFT order; G = 2 pi m / L (solver.py:189-200)
        m = np.fft.fftfreq(self.ng) * self.ng
        self.m1d = m
        self.G1d = 2 * np.pi * m / self.L
        gx, gy, gz = np.meshgrid(self.G1d, self.G1d, self.G1d, indexing="ij")
        self.G = np.stack([gx, gy, gz])
        G2 = gx ** 2 + gy ** 2 + gz ** 2
        with np.errstate(divide="ignore"):
            self.VG = 4 * np.pi / self.Omega / G2
        self.VG[0, 0, 0] = 0.0
        self.coul = self.VG * self.Omega  # 4 pi / G^2 with G=0 -> 0

    # ------------------------------------------------------------------
    def gto1d(self, xp, lextra=0, kpt=None):
        """Lattice-summed 1D factors ``hqc/pbc/gto.py:326-339``.

        Returns g[A, d, i, a, l] = sum_t u^l exp(-alpha_a u^2), u = x_i - R_Ad - t,
        for l = 0 .. lmax + lextra.  With a k-point each term also carries the
        Bloch phase exp(i k_d t) (``eval_pbc_gaussian_power_x_kpt``,
        gto.py:371-388) and the result is complex.
        """
        lm = self.basis.lmax + lextra
        u = self.x1d[None, None, :, None] - xp[:, :, None, None] - self.lat1d[None, None, None, :]
        e = np.exp(-self.basis.alpha[None, None, None, :, None] * (u ** 2)[..., None, :])
        if kpt is not None:
            ph = np.exp(1j * np.asarray(kpt, dtype=float)[:, None] * self.lat1d[None, :])  # (d,t)
            e = e * ph[None, :, None, None, :]
        pw = np.stack([u ** l for l in range(lm + 1)], axis=-1)  # (A,d,i,t,l)
        return np.einsum("Aditl,Adiat->Adial", pw, e)

    def ao_grid(self, xp, deriv=0, atoms=None, kpt=None):
        """AO values on the grid, ``hqc/pbc/gto.py:341-369`` on Rmesh.

        deriv=0: Phi (nao, ng, ng, ng); deriv=1 also grad (3, nao, ...);
        deriv=2 also the hessian (6, nao, ...) ordered xx, yy, zz, xy, xz, yz.
        With a k-point the Bloch sums of gto.py:390-427 (complex).
        """
        b = self.basis
        g = self.gto1d(xp, lextra=deriv, kpt=kpt)  # (A,3,n,a,l)
        dt = complex if kpt is not None else float
        alpha = b.alpha

        def d1(gd, l):
            # d/dx of u^l e^{-a u^2} = l u^{l-1} - 2 a u^{l+1}
            out = -2 * alpha[None, :] * gd[:, :, l + 1]
            if l > 0:
                out = out + l * gd[:, :, l - 1]
            return out

        def d2(gd, l):
            out = -2 * alpha[None, :] * (2 * l + 1) * gd[:, :, l] + 4 * alpha[None, :] ** 2 * gd[:, :, l + 2]
            if l > 1:
                out = out + l * (l - 1) * gd[:, :, l - 2]
            return out

        atoms = list(range(self.n)) if atoms is None else list(atoms)
        nao, ng = len(atoms) * b.nao, self.ng
        phi = np.zeros((nao, ng, ng, ng), dtype=dt)
        grad = np.zeros((3, nao, ng, ng, ng), dtype=dt) if deriv >= 1 else None
        hess = np.zeros((6, nao, ng, ng, ng), dtype=dt) if deriv >= 2 else None
        pairs = [(0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2)]
        for ia, A in enumerate(atoms):
            for k in range(b.nao):
                p = ia * b.nao + k
                pw = [0, 0, 0]
                if b.l[k] == 1:
                    pw[b.cart[k]] = 1
                c = b.coef[k]
                f = [g[A, d][:, :, pw[d]] for d in range(3)]  # (n, a)
                phi[p] = np.einsum("a,ia,ja,ka->ijk", c, f[0], f[1], f[2])
                if deriv >= 1:
                    df = [d1(g[A, d], pw[d]) for d in range(3)]
                    for d in range(3):
                        h = [df[e] if e == d else f[e] for e in range(3)]
                        grad[d, p] = np.einsum("a,ia,ja,ka->ijk", c, h[0], h[1], h[2])
                if deriv >= 2:
                    ddf = [d2(g[A, d], pw[d]) for d in range(3)]
                    for q, (d, e) in enumerate(pairs):
                        if d == e:
                            h = [ddf[z] if z == d else f[z] for z in range(3)]
                        else:
                            h = [df[z] if z in (d, e) else f[z] for z in range(3)]
                        hess[q, p] = np.einsum("a,ia,ja,ka->ijk", c, h[0], h[1], h[2])
        return phi, grad, hess

    # ------------------------------------------------------------------
    def overlap_kinetic(self, xp, deriv=False, kpt=None):
        """Analytic lattice-summed S and T, ``hqc/pbc/solver.py:240-389``.

        The reference obtains p-type integrals by ``jacfwd`` of the s-type
        primitive integral with respect to the centres; here the same
        derivatives are taken in closed form (Hermite derivatives of
        exp(-mu |R+t|^2)).  With deriv=True also returns dS, dT of shape
        (n_atoms, 3, nao, nao): derivative with respect to atom A's position.
        With a k-point every lattice term carries exp(-i k.t)
        (``_eval_intermediate_integral_kpt``, solver.py:257-274) and S, T are
        complex Hermitian.
        """
        b = self.basis
        a = b.alpha
        asum = a[:, None] + a[None, :]
        mu = a[:, None] * a[None, :] / asum
        K = np.pi ** 1.5 / asum ** 1.5
        nb = b.nao
        dt = complex if kpt is not None else float
        phase = None if kpt is None else np.exp(-1j * self.lattice @ np.asarray(kpt, dtype=float))
        S = np.zeros((self.nao, self.nao), dtype=dt)
        T = np.zeros((self.nao, self.nao), dtype=dt)
        dS = np.zeros((self.n, 3, self.nao, self.nao), dtype=dt) if deriv else None
        dT = np.zeros((self.n, 3, self.nao, self.nao), dtype=dt) if deriv else None
        order = 3 if deriv else 2
        for i in range(self.n):
            for j in range(self.n):
                R = xp[i] - xp[j]
                fs, fk = _hermite_lattice(R, self.lattice, mu, K, order, phase)
                Sb, Tb = _sp_block(b, fs, fk, 0)
                S[i * nb:(i + 1) * nb, j * nb:(j + 1) * nb] = Sb
                T[i * nb:(i + 1) * nb, j * nb:(j + 1) * nb] = Tb
                if deriv and i != j:
                    for c in range(3):
                        dSb, dTb = _sp_block(b, fs, fk, 1, c)
                        # d/dR_i = +d/dR, d/dR_j = -d/dR (R = R_i - R_j)
                        dS[i, c, i * nb:(i + 1) * nb, j * nb:(j + 1) * nb] += dSb
                        dT[i, c, i * nb:(i + 1) * nb, j * nb:(j + 1) * nb] += dTb
                        dS[j, c, i * nb:(i + 1) * nb, j * nb:(j + 1) * nb] -= dSb
                        dT[j, c, i * nb:(i + 1) * nb, j * nb:(j + 1) * nb] -= dTb
        return S, T, dS, dT

    # ------------------------------------------------------------------
    def poisson(self, f):
        """Coulomb potential of a periodic grid function (solver.py:616-629).

        v(r) = sum_G 4 pi/(Omega G^2) f(G) e^{iGr}, f(G) = dV sum_r f e^{-iGr};
        this equals ifft(4 pi / G^2 * fft(f)) and drops G = 0.
        """
        ax = tuple(range(f.ndim - 3, f.ndim))
        out = np.fft.ifftn(self.coul * np.fft.fftn(f, axes=ax), axes=ax)
        return out.real if np.isrealobj(f) else out

    def vloc_grid(self, xp):
        """Local potential of the point protons (solver.py:406-408, 427).

        vlocG = -S(G) V(G), S(G) = sum_A e^{-iG.R_A}; by Parseval the
        reference's Re+Im contraction equals dV sum_r v_loc(r) phi_p phi_q.
        """
        ph = [np.exp(-1j * np.outer(xp[:, d], self.G1d)) for d in range(3)]  # (A, n)
        SI = np.einsum("ai,aj,ak->ijk", ph[0], ph[1], ph[2])
        vG = -SI * self.VG
        return (np.fft.ifftn(vG) * self.N).real


def _hermite_lattice(R, lattice, mu, K, order, phase=None):
    """Derivatives up to ``order`` of f(R) = sum_t K e^{-mu|R+t|^2} (overlap)
    and g(R) = sum_t K mu (3 - 2 mu |R+t|^2) e^{-mu|R+t|^2} (kinetic).

    Returns lists fs, fk where index k holds the k-th derivative tensor with
    the primitive-pair axes last: shapes (), (3,), (3,3), (3,3,3) + mu.shape.
    ``phase`` (complex, one per lattice vector) weights each term; the
    derivatives act on the Gaussian only, as the phase does not depend on R.
    """
    u = R[None, :] + lattice  # (t,3)
    u2 = (u ** 2).sum(1)
    E = K[None] * np.exp(-mu[None] * u2[:, None, None])  # (t,a,b)
    if phase is not None:
        E = E * phase[:, None, None]
    I = np.eye(3)
    m = mu[None]
    fs = [E.sum(0)]
    ui = u[:, :, None, None]
    E1 = -2 * m[:, None] * ui * E[:, None]  # (t,3,a,b)
    fs.append(E1.sum(0))
    uu = u[:, :, None] * u[:, None, :]
    E2 = (4 * m[:, None, None] ** 2 * uu[..., None, None] - 2 * m[:, None, None] * I[None, :, :, None, None]) \
        * E[:, None, None]
    fs.append(E2.sum(0))
    if order >= 3:
        uuu = u[:, :, None, None] * u[:, None, :, None] * u[:, None, None, :]
        dsym = (I[None, :, :, None] * u[:, None, None, :] + I[None, :, None, :] * u[:, None, :, None]
                + I[None, None, :, :] * u[:, :, None, None])
        E3 = (-8 * m[:, None, None, None] ** 3 * uuu[..., None, None]
              + 4 * m[:, None, None, None] ** 2 * dsym[..., None, None]) * E[:, None, None, None]
        fs.append(E3.sum(0))
    # kinetic: h = mu q E with q = 3 - 2 mu u^2
    q = 3 - 2 * m * u2[:, None, None]
    q1 = -4 * m[:, None] * ui
    q2 = -4 * m[:, None, None] * I[None, :, :, None, None]
    fk = [(m * q * E).sum(0)]
    fk.append((m[:, None] * (q1 * E[:, None] + q[:, None] * E1)).sum(0))
    t2 = (q2 * E[:, None, None] + q1[:, :, None] * E1[:, None, :] + q1[:, None, :] * E1[:, :, None]
          + q[:, None, None] * E2)
    fk.append((m[:, None, None] * t2).sum(0))
    if order >= 3:
        t3 = (q2[:, :, :, None] * E1[:, None, None, :] + q2[:, :, None, :] * E1[:, None, :, None]
              + q2[:, None, :, :] * E1[:, :, None, None]
              + q1[:, :, None, None] * E2[:, None, :, :] + q1[:, None, :, None] * E2[:, :, None, :]
              + q1[:, None, None, :] * E2[:, :, :, None]
              + q[:, None, None, None] * E3)
        fk.append((m[:, None, None, None] * t3).sum(0))
    return fs, fk


def _sp_block(b, fs, fk, extra, c=None):
    """Contract primitive integrals into the AO block for one atom pair.

    Bra AO p (l, cart a) and ket AO q (l, cart b), ``solver.py:307-321``:
    s-s: f; p_a-s: (1/2alpha_i) d_a f; s-p_b: -(1/2alpha_j) d_b f;
    p_a-p_b: -(1/(4 alpha_i alpha_j)) d_a d_b f (R = bra - ket).
    extra=1 adds one more derivative along c (the force direction).
    """
    nb = b.nao
    ia = 1.0 / b.alpha
    out = []
    for f in (fs, fk):
        M = np.zeros((nb, nb), dtype=np.result_type(f[0], float))
        for p in range(nb):
            for q in range(nb):
                lp, lq = b.l[p], b.l[q]
                k = lp + lq + extra
                idx = []
                if lp:
                    idx.append(b.cart[p])
                if lq:
                    idx.append(b.cart[q])
                if extra:
                    idx.append(c)
                prim = f[k][tuple(idx)] if idx else f[k]
                w = np.outer(b.coef[p], b.coef[q])
                if lp:
                    w = w * (0.5 * ia)[:, None]
                if lq:
                    w = -w * (0.5 * ia)[None, :]
                M[p, q] = np.sum(w * prim)
        out.append(M)
    return out


# ----------------------------------------------------------------------
# Occupations (hqc/tools/smearing.py)
# ----------------------------------------------------------------------
class Occupation:
    """``make_occupation_func`` (smearing.py:4-173), quirks kept."""

    def __init__(self, n, nmo, smearing=False, method="fermi", sigma=0.0, search="bisect",
                 cycle=100, tol=1e-7):
        assert nmo >= n // 2
        self.n, self.nmo, self.smearing = n, nmo, smearing
        self.method, self.sigma, self.search = method, sigma, search
        self.cycle, self.tol = cycle, tol
        if smearing:
            assert method in ("fermi", "gauss")
            from scipy.special import erfinv
            if method == "fermi":
                self.shift = -sigma * np.log(2 * nmo / n - 1)
            else:
                self.shift = -sigma * erfinv(1 - n / nmo)

    def f(self, mu, w):
        if self.method == "fermi":
            return 2 / (np.exp(np.clip((w - mu) / self.sigma, -50, 50)) + 1)
        from scipy.special import erf
        return 0.5 * (1 + erf((mu - w) / self.sigma))

    def dN(self, mu, w):
        """N(mu) - n and its first two derivatives with respect to mu."""
        s = self.sigma
        if self.method == "fermi":
            x = (w - mu) / s
            inside = (x >= -50) & (x <= 50)
            e = np.exp(np.clip(x, -50, 50))
            f = 2 / (e + 1)
            d1 = np.where(inside, 2 * e / (e + 1) ** 2 / s, 0.0)
            d2 = np.where(inside, 2 * e * (e - 1) / (e + 1) ** 3 / s ** 2, 0.0)
        else:
            from scipy.special import erf
            u = (mu - w) / s
            f = 0.5 * (1 + erf(u))
            g = np.exp(-u * u) / np.sqrt(np.pi)
            d1 = g / s
            d2 = -2 * u * g / s ** 2
        return f.sum() - self.n, d1.sum(), d2.sum()

    def mu(self, w):
        if self.search == "bisect":
            return self._bisect(w)
        return self._newton(w)

    def _bisect(self, w):
        """smearing.py:74-102, including its return rule on the sign of mu."""
        tol, cyc = self.tol, self.cycle
        lo, hi = np.min(w) + self.shift, np.max(w) + self.shift
        ylo, yhi, loop = -1.0, 1.0, 0
        while (ylo < -tol) and (yhi > tol) and (loop < cyc):
            mid = (lo + hi) / 2
            ym = self.dN(mid, w)[0]
            lo, hi = (mid, hi) if ym < 0 else (lo, mid)
            ylo, yhi = self.dN(lo, w)[0], self.dN(hi, w)[0]
            loop += 1
        return (lo > -tol) * lo + (hi < tol) * hi + (lo + hi) / 2 * (loop == cyc)

    def _newton(self, w):
        """smearing.py:106-138: Newton minimisation of N(mu)^2."""
        mu0, mu, loop = 1.0, w[self.n // 2], 0
        while abs(mu - mu0) > self.tol and loop < self.cycle:
            N, d1, d2 = self.dN(mu, w)
            g1 = 2 * N * d1
            g2 = 2 * d1 * d1 + 2 * N * d2
            mu0, mu = mu, mu - g1 / abs(g2)
            loop += 1
        return mu

    def __call__(self, w):
        if not self.smearing:
            o = np.zeros(self.nmo)
            o[: self.n // 2] = 2.0
            return o
        return self.f(self.mu(w), w)


def entropy(occ, eps=1e-15):
    """``eval_entropy`` (solver.py:579-590)."""
    h = occ / 2
    with np.errstate(divide="ignore", invalid="ignore"):
        a = np.where(h > eps, h * np.log(np.where(h > eps, h, 1.0)), 0.0)
        b = np.where(1 - h > eps, (1 - h) * np.log(np.where(1 - h > eps, 1 - h, 1.0)), 0.0)
    return -2 * (a.sum() + b.sum())


# ----------------------------------------------------------------------
# The solver
# ----------------------------------------------------------------------
def _tr(A, D):
    """Re tr(A D) (the reference's ``einsum('pq,qp', A, dm).real``)."""
    if np.iscomplexobj(A) or np.iscomplexobj(D):
        return float(np.real(np.sum(A * D.T)))
    return np.sum(A * D)


class Solver:
    """``make_solver`` (solver.py:14-978), streamed form: the Gamma point
    (``hf_gamma`` / ``dft_gamma``) and, when ``solve`` is given a k-point,
    ``hf_kpt`` / ``dft_kpt`` (solver.py:769-962) with complex AOs."""

    def __init__(self, n, L, rs, basis, rcut=24, tol=1e-7, max_cycle=100, grid_length=0.12,
                 diis=True, diis_space=8, diis_start_cycle=1, diis_damp=0.0, dft=False,
                 xc="lda,vwn", smearing=False, smearing_method="fermi", smearing_sigma=0.0,
                 search_method="bisect", search_cycle=100, search_tol=1e-7, n_grid=None,
                 exx_occ_threshold=0.0):
        self.st = Setup(n, L, rs, basis, rcut=rcut, grid_length=grid_length, n_grid=n_grid)
        self.n = n
        self.tol, self.max_cycle = tol, max_cycle
        self.diis, self.space, self.start, self.damp = diis, diis_space, diis_start_cycle, diis_damp
        self.dft = dft
        self.xc = xcmod.Functional(xc) if dft else None
        self.occ = Occupation(n, self.st.nao, smearing, smearing_method, smearing_sigma,
                              search_method, search_cycle, search_tol)
        self.exx_thr = exx_occ_threshold
        self.iterations = 0
        # called with a label after the geometry set-up and after every SCF
        # iteration (timing of a CPU evaluation's pieces); may raise to stop
        self.on_unit = None

    # grid pieces --------------------------------------------------------
    def density(self, D, phi, grad=None):
        """rho = Re sum_pq D_pq phi_p phi_q^* (solver.py:690), as X = D phi^*
        (BLAS); grad rho = 2 Re sum_pq D_pq grad phi_p phi_q^*."""
        shp = phi.shape
        P = phi.reshape(shp[0], -1)
        X = (D @ P.conj())
        rho = np.einsum("pg,pg->g", P, X).real.reshape(shp[1:])
        X = X.reshape(shp)
        if grad is None:
            return rho, None, X
        grho = 2 * np.einsum("dpg,pg->dg", grad.reshape(3, shp[0], -1),
                             X.reshape(shp[0], -1)).real.reshape((3,) + shp[1:])
        return rho, grho, X

    def quadrature(self, w, phi):
        """V_pq = dV sum_r phi_p^* w phi_q (solver.py:693)."""
        P = phi.reshape(phi.shape[0], -1)
        return self.st.dV * ((P.conj() * w.reshape(1, -1)) @ P.T)

    def hartree(self, rho, phi):
        vh = self.st.poisson(rho)
        return self.quadrature(vh, phi), vh

    def exchange(self, D, C, occ, phi, Stilde):
        """K_pq = sum_i f_i dV sum_r (phi_p^* psi_i) W_qi^* + Madelung K0 with
        W_qi = v_H[phi_q^* psi_i] (equals ``exchange(eris + eris0, dm)``,
        solver.py:430-431, 509-524, 604-614; the Gamma point drops the
        conjugations)."""
        st = self.st
        K = np.zeros_like(D)
        for i in range(C.shape[1]):
            if occ[i] <= self.exx_thr:
                continue
            psi = np.einsum("p,pijk->ijk", C[:, i], phi)
            pair = phi.conj() * psi[None]
            W = st.poisson(pair)
            K += occ[i] * st.dV * (pair.reshape(pair.shape[0], -1) @ W.reshape(W.shape[0], -1).conj().T)
        K0 = 4 * np.pi / st.L * MADELUNG_SC * (Stilde @ D @ Stilde)
        return K + K0

    def xc_terms(self, D, phi, grad):
        rho, grho, X = self.density(D, phi, grad if self.xc.gga else None)
        e, vrho, vsig = self.xc.evaluate(rho, None if grho is None else (grho ** 2).sum(0))
        Exc = self.st.dV * e.sum()
        V = self.quadrature(vrho, phi)
        if self.xc.gga:
            u = 2 * vsig[None] * grho  # 2 v_sigma grad rho
            Y = np.einsum("dg,dpg->pg", u.reshape(3, -1), grad.reshape(3, grad.shape[1], -1))
            M = self.st.dV * (Y.conj() @ phi.reshape(phi.shape[0], -1).T)
            V = V + M + M.conj().T
        return Exc, V

    # solve --------------------------------------------------------------
    def setup_geometry(self, xp_rs, kpt=None):
        st = self.st
        xp = np.asarray(xp_rs, dtype=float) * st.rs
        S, T, _, _ = st.overlap_kinetic(xp, kpt=kpt)
        need_grad = self.dft and self.xc.gga
        phi, grad, _ = st.ao_grid(xp, deriv=1 if need_grad else 0, kpt=kpt)
        vloc = st.vloc_grid(xp)
        V = self.quadrature(vloc, phi)
        P = phi.reshape(phi.shape[0], -1)
        return dict(xp=xp, S=S, T=T, phi=phi, grad=grad, vloc=vloc, V=V,
                    Stilde=st.dV * (P.conj() @ P.T))

    def solve(self, xp_rs, kpt=None):
        """One SCF; ``kpt`` (3,) in 1/Bohr selects the k-point solver."""
        g = self.setup_geometry(xp_rs, kpt)
        self._unit("geometry")
        S, T, V, phi, grad = g["S"], g["T"], g["V"], g["phi"], g["grad"]
        cplx = np.iscomplexobj(S)
        w, u = np.linalg.eigh(S)
        v = u @ np.diag(w ** -0.5)
        H = T + V
        occf = self.occ

        def dmat(C, e):
            return C @ np.diag(occf(e)) @ C.conj().T

        def veff(D, C, e):
            rho = self.density(D, phi)[0]
            J, _ = self.hartree(rho, phi)
            if self.dft:
                Exc, Vxc = self.xc_terms(D, phi, grad)
            else:
                K = self.exchange(D, C, occf(e), phi, g["Stilde"])
                Vxc = -0.5 * K
                Exc = 0.5 * _tr(Vxc, D)
            return J, Exc, Vxc

        def diag(F):
            F1 = v.conj().T @ F @ v
            if cplx:
                # jnp.linalg.eigh symmetrises its input: (F1 + F1^H) / 2
                F1 = 0.5 * (F1 + F1.conj().T)
            e, c = np.linalg.eigh(F1)
            return v @ c, e

        C, e = diag(H)
        D = dmat(C, e)
        if self.diis:
            C, e, E, conv = self._diis(H, D, C, e, S, diag, dmat, veff)
        else:
            C, e, E, conv = self._fixed_point(H, D, C, e, diag, dmat, veff)
        D = dmat(C, e)
        J, Exc, _ = veff(D, C, e)
        Ki = _tr(T, D)
        Vep = _tr(V, D)
        Vee = 0.5 * _tr(J, D) + Exc
        Se = entropy(occf(e))
        self.last = dict(g=g, C=C, e=e, D=D, occ=occf(e), E=E, v=v, kpt=kpt)
        return C, D, e * RY, E * RY, Ki * RY, Vep * RY, Vee * RY, Se, conv

    def _unit(self, label):
        if self.on_unit is not None:
            self.on_unit(label)

    def _fixed_point(self, H, D, C, e, diag, dmat, veff):
        """``fixed_point_scf`` (scf.py:21-88)."""
        E0, E1, loop = 0.0, 1.0, 0
        while abs(E1 - E0) > self.tol and loop < self.max_cycle:
            J, Exc, Vxc = veff(D, C, e)
            Enew = 0.5 * _tr(2 * H + J, D) + Exc
            C, e = diag(H + J + Vxc)
            D = dmat(C, e)
            E0, E1, loop = E1, Enew, loop + 1
            self._unit("scf")
        self.iterations = loop
        return C, e, E1, loop != self.max_cycle

    def _diis(self, H, D, C, e, S, diag, dmat, veff):
        """``diis_scf`` (scf.py:90-242)."""
        sp = self.space
        J, _, Vxc = veff(D, C, e)
        F = H + J + Vxc
        err = S @ D @ F - F @ D @ S
        Fk = [F.copy() for _ in range(sp)]
        ek = [err.copy() for _ in range(sp)]
        E0, E1, loop = 0.0, 1.0, 0
        while loop < self.start + sp:
            C, e = diag(Fk[-1])
            D = dmat(C, e)
            J, Exc, Vxc = veff(D, C, e)
            Enew = 0.5 * _tr(2 * H + J, D) + Exc
            F = H + J + Vxc
            err = S @ D @ F - F @ D @ S
            Fk = Fk[1:] + [F]
            ek = ek[1:] + [err]
            E0, E1, loop = E1, Enew, loop + 1
            self._unit("scf")
        E0 = E1 - 1.0
        while ((abs(E1 - E0) > self.tol) or (np.linalg.norm(ek[-1]) > 10 * self.tol)) \
                and loop < self.max_cycle:
            # no conjugation: complex-symmetric B for complex error vectors
            B = np.einsum("imn,jmn->ij", np.array(ek), np.array(ek))
            eta = 1e-12 * (np.trace(B) / sp + 1.0)
            B = B + eta * np.eye(sp)
            h = np.zeros((sp + 1, sp + 1), dtype=B.dtype)
            h[:sp, :sp] = B
            h[:sp, sp] = -1
            h[sp, :sp] = -1
            gvec = np.zeros(sp + 1, dtype=B.dtype)
            gvec[sp] = -1
            c = np.linalg.solve(h, gvec)[:sp]
            Fx = np.einsum("k,kab->ab", c, np.array(Fk))
            Fx = (1 - self.damp) * Fx + self.damp * Fk[-1]
            C, e = diag(Fx)
            D = dmat(C, e)
            J, Exc, Vxc = veff(D, C, e)
            Enew = 0.5 * _tr(2 * H + J, D) + Exc
            F = H + J + Vxc
            err = S @ D @ F - F @ D @ S
            Fk = Fk[1:] + [F]
            ek = ek[1:] + [err]
            E0, E1, loop = E1, Enew, loop + 1
            self._unit("scf")
        self.iterations = loop
        return C, e, E1, loop != self.max_cycle
