"""Oracle: analytic nuclear gradient of the GPW SCF energy (Gamma point and
single k-point).

The reference has no forces (``doc/solver_algorithm.md:1210``); this is a new
FP64 CPU restatement used to check the GPU adjoint (parity unpinned; pinned by
central finite differences of the oracle energy).  For the discrete,
variational energy functional of ``hqc/pbc/solver.py`` (analytic S, T and
grid quadrature for everything else) the total derivative at
self-consistency is

  dE/dR_A = tr(D dT/dR_A) - tr(W dS/dR_A)                 (W = C f eps C^T)
          - 2 dV sum_g V_eff(g) sum_{p in A} grad phi_p(g) (D phi)_p(g)
          + d/dR_A [dV sum_g v_loc(g; R) rho(g)]            (structure factor)
          + GGA and exact-exchange orbital terms,

with Mermin's free energy E - sigma*S in place of E under Fermi smearing.
Units: Hartree per Bohr.  Test infrastructure only.
"""
import numpy as np

from .gpw import MADELUNG_SC


def electronic_gradient(solver):
    """dE/dR (Ha/Bohr), shape (n, 3), for the last ``solver.solve`` call.

    At a k-point (``solver.solve(xp, kpt)``, the single-k ``hf_kpt`` /
    ``dft_kpt`` of solver.py:769-962) the same terms hold for the complex
    Bloch AOs phi^k with X = D conj(phi), traces Re tr(D dT), Re tr(W dS)
    and the grid sums' real parts: rho = Re sum_pq D_pq phi_p conj(phi_q)
    (solver.py:690 as restated in ``Solver.density``) changes by
    2 Re sum_{p in A} dphi_p X_p, and the exchange energy
    -1/4 sum v |gamma(r, r')|^2 by Re sum_{p in A} dphi_p Z_p with
    Z_p = sum_i f_i conj(psi_i) (D W_i)_p, W_ti = v_H[conj(phi_t) psi_i]."""
    st = solver.st
    last = solver.last
    g = last["g"]
    xp = g["xp"]
    kpt = last.get("kpt")
    C, e, D, occ = last["C"], last["e"], last["D"], last["occ"]
    nb = st.nao_atom
    n = st.n
    _, _, dS, dT = st.overlap_kinetic(xp, deriv=True, kpt=kpt)
    W = (C * (occ * e)[None, :]) @ C.conj().T
    grad = np.real(np.einsum("pq,acqp->ac", D, dT) - np.einsum("pq,acqp->ac", W, dS))

    phi = g["phi"]
    X = np.einsum("pq,qijk->pijk", D, phi.conj())
    rho = np.einsum("pijk,pijk->ijk", phi, X).real
    vh = st.poisson(rho)
    veff = g["vloc"] + vh
    gga = solver.dft and solver.xc.gga
    if solver.dft:
        if gga:
            full = st.ao_grid(xp, deriv=1, kpt=kpt)[1]
            grho = 2 * np.einsum("dpijk,pijk->dijk", full, X).real
            _, vrho, vsig = solver.xc.evaluate(rho, (grho ** 2).sum(0))
            u = 2 * vsig[None] * grho
            Psi = np.einsum("dijk,dpijk->pijk", u, full)
            DPsi = np.einsum("pq,qijk->pijk", D, Psi.conj())
            del full
        else:
            _, vrho, _ = solver.xc.evaluate(rho)
        veff = veff + vrho
    else:
        # exact exchange: Z_p = sum_j f_j conj(psi_j) sum_q D_pq W_qj, plus the
        # Madelung term c dV (D S~ D conj(phi))_p
        Z = np.zeros_like(phi)
        for j in range(C.shape[1]):
            if occ[j] <= solver.exx_thr:
                continue
            psi = np.einsum("p,pijk->ijk", C[:, j], phi)
            Wq = st.poisson(phi.conj() * psi[None])
            Z += occ[j] * psi.conj()[None] * np.einsum("pq,qijk->pijk", D, Wq)
        M = D @ g["Stilde"] @ D
        cM = 4 * np.pi / st.L * MADELUNG_SC
        Z += cM * np.einsum("pq,qijk->pijk", M, phi.conj())

    for A in range(n):
        sl = slice(A * nb, (A + 1) * nb)
        _, dphi, hess = st.ao_grid(xp, deriv=2 if gga else 1, atoms=[A], kpt=kpt)
        grad[A] += -2 * st.dV * np.einsum("ijk,cpijk,pijk->c", veff, dphi, X[sl]).real
        if gga:
            # sum_b u_b d_c d_b phi_p ; hessian order xx yy zz xy xz yz
            idx = {(0, 0): 0, (1, 1): 1, (2, 2): 2, (0, 1): 3, (1, 0): 3, (0, 2): 4,
                   (2, 0): 4, (1, 2): 5, (2, 1): 5}
            for c in range(3):
                t = sum(u[b][None] * hess[idx[(c, b)]] for b in range(3))
                grad[A, c] += -2 * st.dV * np.sum(X[sl] * t + dphi[c] * DPsi[sl]).real
        if not solver.dft:
            grad[A] += st.dV * np.einsum("cpijk,pijk->c", dphi, Z[sl]).real

    # structure-factor derivative of the local potential
    F = np.fft.fftn(rho)
    for A in range(n):
        ph = np.einsum("i,j,k->ijk", *[np.exp(-1j * st.G1d * xp[A, d]) for d in range(3)])
        for c in range(3):
            grad[A, c] += np.real(np.sum(1j * st.G[c] * st.VG * ph * st.dV * np.conj(F)))
    return grad
