"""Single-kernel cases at the H54 benchmark shapes, for profiler captures.

    python -m hqc_gb300.profile_cases <case> [--reps R]

Cases (synthetic operands with the benchmark's sizes: 270 AOs, an 81^3 grid,
27 doubly occupied orbitals):

  psi_density   orbital-form density with the gradient (tcgen05, 3xTF32)
  density_D     density-matrix form of the density (tcgen05, 3xTF32)
  quadrature    phi diag(w) phi^T (tcgen05, 3xTF32; symmetric tile set)
  quadrature_gga  Z phi^T + phi Z^T with the PBE operand (the SCF's form)
  eigh_mixed    the mixed-precision eigensolver on a 270 x 270 matrix
  eigh_fp64     the FP64 eigensolver on the same matrix
  exchange      the Hartree-Fock exchange build of one Fock matrix (pair
                planes, column transforms, tcgen05 Gram) at the batched
                workload's H32 dzv 65^3 shape, after one converged mixed SCF

Each case runs its operation ``reps`` times (default 3) after building the
operands, so a profiler can skip the set-up launches and capture the rest.
"""
import argparse

NAO, NG, NOCC = 270, 81, 27


def _operands(gga):
    import torch
    g = torch.Generator(device="cuda").manual_seed(1)
    N = NG ** 3
    ld = (N + 63) // 64 * 64
    phi = torch.zeros(NAO, ld, dtype=torch.float32, device="cuda")
    phi[:, :N] = torch.randn(NAO, N, generator=g, device="cuda") * torch.exp(
        -3 * torch.rand(NAO, N, generator=g, device="cuda"))
    dphi = None
    if gga:
        dphi = torch.zeros(3 * NAO, ld, dtype=torch.float32, device="cuda")
        dphi[:, :N] = torch.randn(3 * NAO, N, generator=g, device="cuda")
    return phi, dphi, N


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["psi_density", "density_D", "quadrature", "quadrature_gga",
                                     "eigh_mixed", "eigh_fp64", "exchange"])
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args(argv)
    import torch
    from hqc_gb300 import _lib
    _lib.load()
    if a.case == "exchange":
        import ctypes
        from hqc_gb300 import make_solver
        from hqc_gb300.workloads import hf_uneven_batch, HF_FERMI_5000K
        xp, L, rs, grid = hf_uneven_batch(256, 3)[-1]
        s = make_solver(xp.shape[0], L, rs, "gth-dzv", precision="mixed", n_grid=grid, tol=1e-7,
                        **HF_FERMI_5000K)
        s(xp)
        lib = _lib.load()
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        for _ in range(a.reps):
            pairs = lib.hqcgb_exchange_rebuild(s.plan.handle, st)
        print(f"exchange: {pairs} AO-orbital pairs per build")
    elif a.case.startswith("eigh"):
        g = torch.Generator(device="cuda").manual_seed(2)
        M = torch.randn(NAO, NAO, dtype=torch.float64, device="cuda", generator=g)
        M = M + M.T
        fn = _lib.eigh_mixed if a.case == "eigh_mixed" else _lib.eigh
        for _ in range(a.reps):
            fn(M)
    elif a.case == "psi_density":
        phi, dphi, N = _operands(True)
        C = torch.randn(NAO, NAO, dtype=torch.float64, device="cuda") / NAO ** 0.5
        occ = torch.zeros(NAO, dtype=torch.float64, device="cuda")
        occ[:NOCC] = 2.0
        for _ in range(a.reps):
            _lib.tc_orbital_density(phi, C, occ, N, NOCC, dphi)
    elif a.case == "density_D":
        phi, _, N = _operands(False)
        D = torch.randn(NAO, NAO, device="cuda")
        D = 0.5 * (D + D.T)
        for _ in range(a.reps):
            _lib.tc_density(phi, D, N, drain=1)
    elif a.case == "quadrature_gga":
        phi, dphi, N = _operands(True)
        ld = phi.shape[1]
        w = torch.zeros(ld, dtype=torch.float32, device="cuda")
        w[:N] = torch.rand(N, device="cuda")
        u = torch.zeros(3, ld, dtype=torch.float32, device="cuda")
        u[:, :N] = torch.randn(3, N, device="cuda")
        for _ in range(a.reps):
            _lib.tc_quadrature_gga(phi, dphi, w, u, 1e-3, N, drain=4)
    else:
        phi, _, N = _operands(False)
        w = torch.zeros(phi.shape[1], dtype=torch.float32, device="cuda")
        w[:N] = torch.rand(N, device="cuda")
        for _ in range(a.reps):
            _lib.tc_quadrature(phi, w, drain=4)
    torch.cuda.synchronize()
    print(f"{a.case}: {a.reps} runs ok")


if __name__ == "__main__":
    main()
