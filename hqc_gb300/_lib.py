"""ctypes binding of ``libhqcgb.so`` (the C ABI declared in ``include/hqcgb.h``).

The product has no CPU fallback: if the library is missing or cannot be
loaded, every entry point raises.  Build it with ``python -m hqc_gb300.build``
(``__graft_entry__.build()`` does the same).
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhqcgb.so")

c_double_p = ctypes.POINTER(ctypes.c_double)
c_int_p = ctypes.POINTER(ctypes.c_int)

STATUS = {0: "OK", 1: "NOT_CONVERGED", 2: "BAD_ARG", 3: "CUDA_ERROR", 4: "EIG_FAIL", 5: "NAN",
          6: "NO_STATE"}
XC = {"lda,": 0, "lda,vwn": 1, "lda,hl": 2, "lda,hl71": 2, "lda,bh": 3, "lda,bh72": 3,
      "lda,gl": 4, "lda,gl77": 4, "pbe": 10, "gga_x_pbe,gga_c_pbe": 10, "pbe,pbe": 10}


class Params(ctypes.Structure):
    _fields_ = [
        ("n_atoms", ctypes.c_int), ("n_grid", ctypes.c_int), ("L", ctypes.c_double),
        ("nao_atom", ctypes.c_int), ("n_prim", ctypes.c_int),
        ("alpha", c_double_p), ("coef", c_double_p), ("ao_l", c_int_p), ("ao_cart", c_int_p),
        ("n_lat1d", ctypes.c_int), ("lat1d", c_double_p),
        ("n_lattice", ctypes.c_int), ("lattice", c_double_p),
        ("dft", ctypes.c_int), ("xc", ctypes.c_int), ("smearing", ctypes.c_int),
        ("smearing_method", ctypes.c_int), ("smearing_sigma", ctypes.c_double),
        ("search_method", ctypes.c_int), ("search_cycle", ctypes.c_int),
        ("search_tol", ctypes.c_double), ("tol", ctypes.c_double), ("max_cycle", ctypes.c_int),
        ("diis", ctypes.c_int), ("diis_space", ctypes.c_int), ("diis_start_cycle", ctypes.c_int),
        ("diis_damp", ctypes.c_double), ("precision", ctypes.c_int),
        ("exx_occ_threshold", ctypes.c_double), ("want_forces", ctypes.c_int),
    ]


class ScfOut(ctypes.Structure):
    _fields_ = [("mo_coeff", ctypes.c_void_p), ("dm", ctypes.c_void_p), ("bands", ctypes.c_void_p),
                ("energies", ctypes.c_void_p), ("converged", ctypes.c_void_p),
                ("iterations", ctypes.c_void_p), ("free_energy", ctypes.c_void_p)]


EXPORTS = ("hqcgb_plan_create", "hqcgb_plan_destroy", "hqcgb_scf", "hqcgb_scf_batch",
           "hqcgb_forces", "hqcgb_ewald", "hqcgb_plan_query", "hqcgb_last_error",
           "hqcgb_launch_count", "hqcgb_profile", "hqcgb_stage_stats", "hqcgb_eigh",
           "hqcgb_eigh_noalloc", "hqcgb_eigh_mixed", "hqcgb_tc_quadrature", "hqcgb_tc_density",
           "hqcgb_tc_orbital_density", "hqcgb_plan_set_concurrency", "hqcgb_pes_batch",
           "hqcgb_ao_points", "hqcgb_slater", "hqcgb_kplan_create", "hqcgb_kplan_destroy",
           "hqcgb_scf_kpt", "hqcgb_scf_kpt_batch", "hqcgb_kplan_query", "hqcgb_eigh_herm",
           "hqcgb_ao_points_kpt", "hqcgb_slater_kpt", "hqcgb_overlap", "hqcgb_coulomb_energy",
           "hqcgb_tc_quadrature_gga", "hqcgb_diis_coefficients",
           "hqcgb_tc_quad_tiles", "hqcgb_batch_create", "hqcgb_batch_destroy", "hqcgb_batch_run",
           "hqcgb_exchange_rebuild", "hqcgb_tune_set", "hqcgb_tune_get", "hqcgb_forces_kpt",
           "hqcgb_pes_kpt_batch")
N_STAGES = 15

_lib = None


class HqcgbError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"hqcgb {STATUS.get(status, status)}: {msg}")
        self.status = status


def load():
    """Load the engine; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build the CUDA engine with "
                           "`python -m hqc_gb300.build` (there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    lib.hqcgb_plan_create.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_void_p)]
    lib.hqcgb_plan_destroy.argtypes = [ctypes.c_void_p]
    lib.hqcgb_scf.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ScfOut),
                              ctypes.c_void_p]
    lib.hqcgb_scf_batch.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                    ctypes.POINTER(ScfOut), ctypes.c_void_p]
    lib.hqcgb_forces.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_plan_set_concurrency.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.hqcgb_ao_points.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                    c_int_p, c_int_p, ctypes.c_int, c_double_p, ctypes.c_void_p,
                                    ctypes.c_longlong, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p]
    lib.hqcgb_slater.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                 c_int_p, c_int_p, ctypes.c_int, c_double_p, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                 c_int_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_ao_points_kpt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p,
                                        c_double_p, c_int_p, c_int_p, ctypes.c_int, c_double_p,
                                        c_double_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_slater_kpt.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                     c_int_p, c_int_p, ctypes.c_int, c_double_p, c_double_p,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int, c_int_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_overlap.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p,
                                  c_int_p, c_int_p, ctypes.c_int, c_double_p, ctypes.c_int,
                                  ctypes.c_void_p, c_double_p, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p]
    lib.hqcgb_coulomb_energy.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                         c_int_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_pes_batch.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                    ctypes.POINTER(ScfOut), ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_batch_create.argtypes = [ctypes.POINTER(Params), ctypes.c_double, ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_void_p)]
    lib.hqcgb_batch_destroy.argtypes = [ctypes.c_void_p]
    lib.hqcgb_tune_set.argtypes = [ctypes.c_char_p, ctypes.c_longlong]
    lib.hqcgb_tune_get.argtypes = [ctypes.c_char_p]
    lib.hqcgb_tune_get.restype = ctypes.c_longlong
    lib.hqcgb_exchange_rebuild.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_exchange_rebuild.restype = ctypes.c_longlong
    lib.hqcgb_batch_run.argtypes = [ctypes.c_void_p, ctypes.c_int, c_int_p, c_int_p, c_double_p,
                                    ctypes.c_void_p, ctypes.POINTER(ScfOut), ctypes.c_void_p,
                                    ctypes.c_void_p]
    lib.hqcgb_ewald.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_void_p]
    lib.hqcgb_plan_query.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p,
                                     ctypes.c_size_t, ctypes.c_void_p]
    lib.hqcgb_plan_query.restype = ctypes.c_longlong
    lib.hqcgb_kplan_create.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(ctypes.c_void_p)]
    lib.hqcgb_kplan_destroy.argtypes = [ctypes.c_void_p]
    lib.hqcgb_scf_kpt.argtypes = [ctypes.c_void_p, ctypes.c_void_p, c_double_p,
                                  ctypes.POINTER(ScfOut), ctypes.c_void_p]
    lib.hqcgb_scf_kpt_batch.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, c_double_p,
                                        ctypes.POINTER(ScfOut), ctypes.c_void_p]
    lib.hqcgb_forces_kpt.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_pes_kpt_batch.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, c_double_p,
                                        ctypes.POINTER(ScfOut), ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_kplan_query.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p,
                                      ctypes.c_size_t, ctypes.c_void_p]
    lib.hqcgb_kplan_query.restype = ctypes.c_longlong
    lib.hqcgb_diis_coefficients.argtypes = [ctypes.c_int, c_double_p, c_double_p]
    lib.hqcgb_tc_quad_tiles.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_int_p, c_int_p, c_int_p]
    lib.hqcgb_eigh_herm.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                    ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_last_error.restype = ctypes.c_char_p
    lib.hqcgb_launch_count.argtypes = [ctypes.c_int]
    lib.hqcgb_launch_count.restype = ctypes.c_longlong
    lib.hqcgb_profile.argtypes = [ctypes.c_int]
    lib.hqcgb_eigh.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                               ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_tc_quadrature.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_longlong,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_tc_quadrature_gga.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_longlong] + \
        [ctypes.c_void_p] * 4 + [ctypes.c_float, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_tc_density.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_longlong,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_tc_orbital_density.argtypes = [ctypes.c_int, ctypes.c_longlong, ctypes.c_longlong] + \
        [ctypes.c_void_p] * 4 + [ctypes.c_int, ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 3
    lib.hqcgb_eigh_mixed.argtypes = [ctypes.c_int] + [ctypes.c_void_p] * 4
    lib.hqcgb_eigh_noalloc.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p]
    lib.hqcgb_stage_stats.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_char_p),
                                      ctypes.POINTER(ctypes.c_longlong),
                                      ctypes.POINTER(ctypes.c_double)]
    for name in EXPORTS:
        getattr(lib, name)
    _lib = lib
    return lib


def check(status, allow=(0,)):
    if status not in allow:
        msg = load().hqcgb_last_error().decode(errors="replace")
        raise HqcgbError(status, msg)
    return status


def stage_stats():
    """{stage name: (launches, device ms)} since the last profile(1)."""
    lib = load()
    out = {}
    for k in range(N_STAGES):
        name = ctypes.c_char_p()
        cnt = ctypes.c_longlong()
        ms = ctypes.c_double()
        check(lib.hqcgb_stage_stats(k, ctypes.byref(name), ctypes.byref(cnt), ctypes.byref(ms)))
        out[name.value.decode()] = (cnt.value, ms.value)
    return out


def profile(enable):
    check(load().hqcgb_profile(int(enable)))


def eigh(A):
    """FP64 symmetric eigendecomposition on the GPU: (w ascending, V columns).

    ``A`` is a float64 CUDA tensor of shape (n, n) or (batch, n, n)."""
    import torch
    lib = load()
    A = A.contiguous()
    single = A.dim() == 2
    A3 = A.unsqueeze(0) if single else A
    b, n, _ = A3.shape
    w = torch.empty(b, n, dtype=torch.float64, device=A.device)
    V = torch.empty(b, n, n, dtype=torch.float64, device=A.device)
    st = ctypes.c_void_p(torch.cuda.current_stream(A.device).cuda_stream)
    check(lib.hqcgb_eigh(n, b, ctypes.c_void_p(A3.data_ptr()), ctypes.c_void_p(w.data_ptr()),
                         ctypes.c_void_p(V.data_ptr()), st))
    return (w[0], V[0]) if single else (w, V)


def eigh_herm(A):
    """FP64 complex Hermitian eigendecomposition on the GPU: (w ascending,
    V columns).  ``A`` is a complex128 CUDA tensor (n, n) or (batch, n, n);
    both triangles are read, so it must be Hermitian."""
    import torch
    lib = load()
    A = A.contiguous()
    if A.dtype != torch.complex128:
        raise TypeError("eigh_herm expects a complex128 tensor")
    single = A.dim() == 2
    A3 = A.unsqueeze(0) if single else A
    b, n, _ = A3.shape
    w = torch.empty(b, n, dtype=torch.float64, device=A.device)
    V = torch.empty(b, n, n, dtype=torch.complex128, device=A.device)
    st = ctypes.c_void_p(torch.cuda.current_stream(A.device).cuda_stream)
    check(lib.hqcgb_eigh_herm(n, b, ctypes.c_void_p(A3.data_ptr()), ctypes.c_void_p(w.data_ptr()),
                              ctypes.c_void_p(V.data_ptr()), st))
    return (w[0], V[0]) if single else (w, V)


def eigh_mixed(A):
    """The mixed-precision eigensolver (FP32 solve + FP64 refinement) on one
    (n, n) float64 CUDA matrix: (w ascending, V columns)."""
    import torch
    lib = load()
    A = A.contiguous()
    n = A.shape[0]
    w = torch.empty(n, dtype=torch.float64, device=A.device)
    V = torch.empty(n, n, dtype=torch.float64, device=A.device)
    st = ctypes.c_void_p(torch.cuda.current_stream(A.device).cuda_stream)
    check(lib.hqcgb_eigh_mixed(n, ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(w.data_ptr()),
                               ctypes.c_void_p(V.data_ptr()), st))
    return w, V


EIGH_NOALLOC_MAX_N = 320


def eigh_noalloc(A, w=None, V=None):
    """``eigh`` of one (n, n) float64 CUDA matrix through ``hqcgb_eigh_noalloc``.

    The engine call allocates nothing (its scratch is a static device array
    shared by all calls on the device, n <= 320).  Callers that cannot
    allocate pass preallocated ``w`` (n,) and ``V`` (n, n) buffers; otherwise
    they are created here, on the torch side."""
    import torch
    lib = load()
    A = A.contiguous()
    n = A.shape[0]
    if w is None:
        w = torch.empty(n, dtype=torch.float64, device=A.device)
    if V is None:
        V = torch.empty(n, n, dtype=torch.float64, device=A.device)
    st = ctypes.c_void_p(torch.cuda.current_stream(A.device).cuda_stream)
    check(lib.hqcgb_eigh_noalloc(n, ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(w.data_ptr()),
                                 ctypes.c_void_p(V.data_ptr()), st))
    return w, V


def quad_tiles(nao, sym=True):
    """Tile plan of the tensor-core quadrature (host only): an int array
    (count, 7) of {kind, mt, nt, arow, brow, nb, swap} rows and the number of
    kernel launches before the reduce."""
    import numpy as np
    lib = load()
    count, launches = ctypes.c_int(0), ctypes.c_int(0)
    check(lib.hqcgb_tc_quad_tiles(nao, int(sym), 0, None, ctypes.byref(count), ctypes.byref(launches)))
    out = np.zeros((count.value, 7), dtype=np.int32)
    check(lib.hqcgb_tc_quad_tiles(nao, int(sym), count.value, out.ctypes.data_as(c_int_p),
                                  ctypes.byref(count), ctypes.byref(launches)))
    return out, launches.value


def tc_quadrature(phi32, w32, nsplit=2, drain=2):
    """M = phi diag(w) phi^T on the tensor cores; phi32 (nao, ld), w32 (ld,) fp32 CUDA."""
    import torch
    lib = load()
    nao, ld = phi32.shape
    M = torch.empty(nao, nao, dtype=torch.float64, device=phi32.device)
    st = ctypes.c_void_p(torch.cuda.current_stream(phi32.device).cuda_stream)
    check(lib.hqcgb_tc_quadrature(nao, ld, ld, ctypes.c_void_p(phi32.data_ptr()),
                                  ctypes.c_void_p(w32.data_ptr()), nsplit, drain,
                                  ctypes.c_void_p(M.data_ptr()), st))
    return M


def tc_quadrature_gga(phi32, dphi32, w32, u32, dV, N=None, drain=4):
    """M = Z phi^T + phi Z^T, Z = 0.5 w phi + dV u . grad phi (fp32 operands on
    the device, row stride a multiple of 32): (nao, nao) float64."""
    import torch
    lib = load()
    nao, ld = phi32.shape
    N = ld if N is None else N
    M = torch.empty(nao, nao, dtype=torch.float64, device=phi32.device)
    st = ctypes.c_void_p(torch.cuda.current_stream(phi32.device).cuda_stream)
    check(lib.hqcgb_tc_quadrature_gga(nao, N, ld, ctypes.c_void_p(phi32.data_ptr()),
                                      ctypes.c_void_p(dphi32.data_ptr()), ctypes.c_void_p(w32.data_ptr()),
                                      ctypes.c_void_p(u32.data_ptr()), float(dV), int(drain),
                                      ctypes.c_void_p(M.data_ptr()), st))
    return M


def tc_density(phi32, D32, N=None, nsplit=2, drain=1):
    """rho[g] = sum_pq D[p][q] phi[p][g] phi[q][g] on the tensor cores."""
    import torch
    lib = load()
    nao, ld = phi32.shape
    N = ld if N is None else N
    rho = torch.empty(N, dtype=torch.float64, device=phi32.device)
    st = ctypes.c_void_p(torch.cuda.current_stream(phi32.device).cuda_stream)
    check(lib.hqcgb_tc_density(nao, N, ld, ctypes.c_void_p(phi32.data_ptr()),
                               ctypes.c_void_p(D32.data_ptr()), nsplit, drain,
                               ctypes.c_void_p(rho.data_ptr()), st))
    return rho


def tc_orbital_density(phi32, C, occ, N=None, nuse=None, dphi32=None, drain=1):
    """rho = sum_k occ_k (sum_p C[p,k] phi_p)^2 (and grad rho with dphi32) on
    the tensor cores; phi32 (nao, ld) fp32, C (nao, nmo) and occ (nmo,) fp64."""
    import torch
    lib = load()
    nao, ld = phi32.shape
    N = ld if N is None else N
    nmo = C.shape[1]
    nuse = nmo if nuse is None else nuse
    dev = phi32.device
    rho = torch.empty(N, dtype=torch.float64, device=dev)
    grho = torch.empty(3, N, dtype=torch.float64, device=dev) if dphi32 is not None else None
    C = C.contiguous()
    occ = occ.contiguous()
    st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    check(lib.hqcgb_tc_orbital_density(
        nao, N, ld, ctypes.c_void_p(phi32.data_ptr()),
        ctypes.c_void_p(dphi32.data_ptr() if dphi32 is not None else 0),
        ctypes.c_void_p(C.data_ptr()), ctypes.c_void_p(occ.data_ptr()), nmo, nuse, drain,
        ctypes.c_void_p(rho.data_ptr()), ctypes.c_void_p(grho.data_ptr() if grho is not None else 0), st))
    return rho if grho is None else (rho, grho)
