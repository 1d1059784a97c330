"""``make_lcao`` (hqc/pbc/lcao.py:11-103): ``lcao(xp)`` -> (mo_coeff, bands, E).

Same as ``make_solver`` except the default chemical-potential search is
Newton (lcao.py:26) and only three outputs are returned; ``gamma=False``
gives ``lcao(xp, kpt)`` (lcao_kpt, lcao.py:80-94).
"""
from .solver import make_solver


def make_lcao(n, L, rs, basis, rcut=24, tol=1e-7, max_cycle=100, grid_length=0.12, diis=True,
              diis_space=8, diis_start_cycle=1, diis_damp=0., use_jit=True, dft=False,
              xc='lda,vwn', smearing=False, smearing_method='fermi', smearing_sigma=0.,
              search_method='newton', search_cycle=100, search_tol=1e-7, gamma=True,
              precision='fp64', forces=False, n_grid=None, exx_occ_threshold=0.0, concurrency=1):
    solver = make_solver(n, L, rs, basis, rcut=rcut, tol=tol, max_cycle=max_cycle,
                         grid_length=grid_length, diis=diis, diis_space=diis_space,
                         diis_start_cycle=diis_start_cycle, diis_damp=diis_damp, use_jit=use_jit,
                         dft=dft, xc=xc, smearing=smearing, smearing_method=smearing_method,
                         smearing_sigma=smearing_sigma, search_method=search_method,
                         search_cycle=search_cycle, search_tol=search_tol, gamma=gamma,
                         precision=precision, forces=forces, n_grid=n_grid,
                         exx_occ_threshold=exx_occ_threshold, concurrency=concurrency)

    if gamma:
        def lcao(xp):
            mo_coeff, _, bands, E, _, _, _, _, _ = solver(xp)
            return mo_coeff, bands, E
    else:
        def lcao(xp, kpt):
            mo_coeff, _, bands, E, _, _, _, _, _ = solver(xp, kpt)
            return mo_coeff, bands, E

    lcao.solver = solver
    return lcao
