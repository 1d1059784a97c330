"""``make_pes``: potential energy surface factory (hqc/pbc/pes.py:10-152).

``pes(xp)`` returns E + Vpp in Rydberg (mode 'default') or the 7-tuple
(E + Vpp, Ki, Vep, Vee, Vpp, Se, converged) in mode 'dev'.  With
``forces=True``, ``pes.value_and_grad(xp)`` returns a matching pair
(F + Vpp, d(F + Vpp)/dxp) in Rydberg (per rs unit) from the engine's adjoint
(absent from the reference).  F is the free energy E - sigma S whose exact
gradient the adjoint computes: without smearing F = E, so the value is
``pes(xp)``; with smearing S is the entropy that makes the smeared
occupations stationary (Fermi: the reference's Se; Gaussian:
sum exp(-x^2) / (2 sqrt(pi))), while ``pes(xp)`` keeps the reference's
internal energy E (hqc/pbc/pes.py:86), whose gradient would need the
occupations' response.
``gamma=False`` gives ``pes(xp, kpt)`` (pes_kpt / pes_dev_kpt,
pes.py:88-137) and, with ``forces=True``, ``pes.value_and_grad(xp, kpt)``:
the single-k free energy plus Vpp and its gradient at the fixed k-point.
"""
import numpy as np
import torch

from .solver import make_solver, RY
from .potential import potential_energy_pp_and_grad


def make_pes(n, L, rs, basis, rcut=24, tol=1e-7, max_cycle=100, grid_length=0.12, diis=True,
             diis_space=8, diis_start_cycle=1, diis_damp=0., use_jit=True, dft=False,
             xc='lda,vwn', smearing=False, smearing_method='fermi', smearing_sigma=0.,
             search_method='bisect', search_cycle=100, search_tol=1e-7, gamma=True, Gmax=15,
             kappa=10, mode='default', precision='fp64', forces=False, n_grid=None,
             exx_occ_threshold=0.0, concurrency=1):
    if mode not in ("default", "dev"):
        raise ValueError(f"Invalid mode: {mode}.")
    solver = make_solver(n, L, rs, basis, rcut=rcut, tol=tol, max_cycle=max_cycle,
                         grid_length=grid_length, diis=diis, diis_space=diis_space,
                         diis_start_cycle=diis_start_cycle, diis_damp=diis_damp, use_jit=use_jit,
                         dft=dft, xc=xc, smearing=smearing, smearing_method=smearing_method,
                         smearing_sigma=smearing_sigma, search_method=search_method,
                         search_cycle=search_cycle, search_tol=search_tol, gamma=gamma,
                         precision=precision, forces=forces, n_grid=n_grid,
                         exx_occ_threshold=exx_occ_threshold, concurrency=concurrency)

    def _arr(xp):
        return xp if isinstance(xp, torch.Tensor) else np.asarray(xp, dtype=np.float64)

    def _vpp(xp):
        """Ewald energy and gradient of one configuration or a batch."""
        if xp.ndim == 3:
            pairs = [potential_energy_pp_and_grad(x, L, rs, kappa=kappa, Gmax=Gmax) for x in xp]
            return torch.stack([e for e, _ in pairs]), torch.stack([g for _, g in pairs])
        return potential_energy_pp_and_grad(xp, L, rs, kappa=kappa, Gmax=Gmax)

    def pes(xp, *kpt):
        if gamma == bool(kpt):
            raise TypeError("pes(xp) at the Gamma point, pes(xp, kpt) with gamma=False")
        xp = _arr(xp)
        _, _, _, E, Ki, Vep, Vee, Se, conv = solver(xp, *kpt)
        Vpp, _ = _vpp(xp)
        if mode == "dev":
            return E + Vpp, Ki, Vep, Vee, Vpp, Se, conv
        return E + Vpp

    def value_and_grad(xp, *kpt):
        """(F + Vpp, d(F + Vpp)/dxp), F = E - sigma S (E without smearing); a
        batch (B, n, 3) gives (B,) and (B, n, 3).  With gamma=False the
        k-point comes second: a batch of xp and/or kpt (B, 3) broadcasts."""
        if gamma == bool(kpt):
            raise TypeError("value_and_grad(xp) at the Gamma point, value_and_grad(xp, kpt) with gamma=False")
        xp = _arr(xp)
        if kpt:
            out = solver.batch(xp, kpt[0], forces=True)
            B = out["grad"].shape[0]
            xb = xp if xp.ndim == 3 else (xp.unsqueeze(0) if isinstance(xp, torch.Tensor) else xp[None])
            Vpp, gpp = _vpp(xb)
            if xb.shape[0] != B:
                Vpp, gpp = Vpp.expand(B), gpp.expand(B, n, 3)
            F, g = out["free_energy"] * RY + Vpp, out["grad"] + gpp
            batched = xp.ndim == 3 or np.asarray(kpt[0].cpu() if isinstance(kpt[0], torch.Tensor)
                                                 else kpt[0]).ndim == 2
            return (F, g) if batched else (F[0], g[0])
        if xp.ndim == 3:
            out = solver.batch(xp, forces=True, full=False)
            Vpp, gpp = _vpp(xp)
            return out["free_energy"] * RY + Vpp, out["grad"] * (RY * rs) + gpp
        solver(xp)
        Vpp, gpp = _vpp(xp)
        return solver.free_energy + Vpp, solver.grad() + gpp

    pes.solver = solver
    pes.value_and_grad = value_and_grad
    return pes
