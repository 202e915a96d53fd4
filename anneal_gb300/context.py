"""Python handle on one solver context of the CUDA library (one voxel grid).

Arguments are torch CUDA tensors used as plain device buffers; each method checks dtype,
device, size and contiguity, passes raw pointers and the current CUDA stream through the
C ABI, and raises ``NativeError`` on a non-zero status.
"""
import ctypes

import numpy as np
import torch

from . import _native as N

_F32, _F64, _U8 = torch.float32, torch.float64, torch.uint8


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("anneal_gb300 runs on a CUDA GPU (sm_103a); none is visible")


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _chk(t, dtype, numel, name):
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name}: expected a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name}: expected {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name}: tensor must be contiguous")
    if numel is not None and t.numel() != numel:
        raise ValueError(f"{name}: expected {numel} values, got {t.numel()}")
    return t


class Context:
    """A solver context: the grid, the free-DOF masks, the multigrid hierarchy and the
    workspaces live on the GPU until ``close()``."""

    def __init__(self, shape, h=1.0, nu=0.3, fp64=False, nrhs=1):
        require_cuda()
        self.lib = N.load()
        self.shape = tuple(int(s) for s in shape)
        nx, ny, nz = self.shape
        self.ne = nx * ny * nz
        self.nn = (nx + 1) * (ny + 1) * (nz + 1)
        self.ndof = 3 * self.nn
        self.h = float(h)
        self.nu = float(nu)
        self.fp64 = bool(fp64)
        self.vdtype = _F64 if fp64 else _F32
        # right-hand-side slots: an FP32 solve of 1 < nrhs <= this many cases runs them together
        self.nrhs = 1 if fp64 else int(nrhs)
        if not 1 <= self.nrhs <= 255:
            raise ValueError("nrhs must be in 1..255")
        flags = N.ANL_FLAG_FP64 if fp64 else N.ANL_FLAG_RHS(self.nrhs)
        h_ = ctypes.c_void_p()
        N.check(self.lib.anl_ctx_create(ctypes.byref(h_), nx, ny, nz, self.h, self.nu, flags), "anl_ctx_create")
        self._h = h_
        self.nfree = None
        self.filter_r = None

    # -- life cycle
    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self.lib.anl_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- domain
    def set_domain(self, active, fixed):
        _chk(active, _U8, self.ne, "active")
        _chk(fixed, _U8, self.ndof, "fixed")
        nfree = ctypes.c_int64(0)
        N.check(self.lib.anl_set_domain(self._h, _p(active), _p(fixed), ctypes.byref(nfree), _stream()),
                "anl_set_domain")
        self.nfree = int(nfree.value)
        return self.nfree

    def free_mask(self):
        out = torch.empty(self.ndof, dtype=_U8, device="cuda")
        N.check(self.lib.anl_free_mask(self._h, _p(out), _stream()), "anl_free_mask")
        return out

    # -- operator and solve
    def apply_K(self, escale, u, y):
        _chk(escale, _F32, self.ne, "escale")
        _chk(u, self.vdtype, self.ndof, "u")
        _chk(y, self.vdtype, self.ndof, "y")
        N.check(self.lib.anl_apply_K(self._h, _p(escale), _p(u), _p(y), _stream()), "anl_apply_K")

    def solve(self, escale, F, X, rtol, maxiter=2000, rebuild=True):
        """F, X: (nrhs, ndof) float64; X holds the initial guesses. Returns (status, iters,
        relres) without raising on MAXITER / NONFINITE / BREAKDOWN / SINGULAR / STAGNATION
        (the caller decides: the first four mean the part is not properly supported or the
        solve failed; STAGNATION asks for the FP64 context to finish an FP32 solve)."""
        _chk(escale, _F32, self.ne, "escale")
        nrhs = F.shape[0] if F.dim() == 2 else 1
        _chk(F, _F64, nrhs * self.ndof, "F")
        _chk(X, _F64, nrhs * self.ndof, "X")
        iters = (ctypes.c_int * nrhs)()
        relres = (ctypes.c_double * nrhs)()
        st = self.lib.anl_solve(self._h, _p(escale), _p(F), _p(X), nrhs, float(rtol), int(maxiter),
                                1 if rebuild else 0, iters, relres, _stream())
        if st not in (N.ANL_OK, N.ANL_ERR_MAXITER, N.ANL_ERR_NONFINITE, N.ANL_ERR_BREAKDOWN,
                      N.ANL_ERR_SINGULAR, N.ANL_ERR_STAGNATION):
            N.check(st, "anl_solve")
        return st, list(iters), list(relres)

    def solve_status(self, k):
        """Status of case k in the last solve (anl_solve returns the first non-OK one)."""
        return int(self.lib.anl_solve_status(self._h, int(k)))

    def profile_apply(self, u, y, reps):
        """Mean milliseconds per launch of the level-0 K u kernel (element scales from the
        last apply_K / solve)."""
        _chk(u, self.vdtype, self.ndof, "u")
        _chk(y, self.vdtype, self.ndof, "y")
        ms = ctypes.c_double(0.0)
        N.check(self.lib.anl_profile_apply(self._h, _p(u), _p(y), int(reps), ctypes.byref(ms), _stream()),
                "anl_profile_apply")
        return float(ms.value)

    def profile_pass(self, pass_id, reps):
        """Mean milliseconds per launch of a finest-level solve pass (0 K u, 1 K u with u.Ku,
        2 residual, 3 last Chebyshev step of a sweep, 4 fused first two Chebyshev steps, 5 first step
        of the post-smoothing sweep); after a solve."""
        ms = ctypes.c_double(0.0)
        N.check(self.lib.anl_profile_pass(self._h, int(pass_id), int(reps), ctypes.byref(ms), _stream()),
                "anl_profile_pass")
        return float(ms.value)

    def mg_info(self):
        """[(element dims, lambda_max estimate)] per multigrid level."""
        nlev = ctypes.c_int(0)
        dims = (ctypes.c_int * 48)()
        lmax = (ctypes.c_double * 16)()
        N.check(self.lib.anl_mg_info(self._h, ctypes.byref(nlev), dims, lmax), "anl_mg_info")
        return [((dims[3 * l], dims[3 * l + 1], dims[3 * l + 2]), lmax[l]) for l in range(nlev.value)]

    def dot(self, a, b):
        _chk(a, _F64, self.ndof, "a")
        _chk(b, _F64, self.ndof, "b")
        out = ctypes.c_double(0.0)
        N.check(self.lib.anl_dot(self._h, _p(a), _p(b), ctypes.byref(out), _stream()), "anl_dot")
        return float(out.value)

    # -- sensitivity
    def element_energy(self, u, ce):
        _chk(u, _F64, self.ndof, "u")
        _chk(ce, _F32, self.ne, "ce")
        N.check(self.lib.anl_element_energy(self._h, _p(u), _p(ce), _stream()), "anl_element_energy")

    def element_stress(self, u, E_material, sig=None, vm=None):
        """E_material: float64 CUDA tensor (ne) or a number; sig (ne, 6) / vm (ne) float64."""
        _chk(u, _F64, self.ndof, "u")
        if torch.is_tensor(E_material):
            _chk(E_material, _F64, self.ne, "E_material")
            em, es = _p(E_material), 0.0
        else:
            em, es = None, float(E_material)
        N.check(self.lib.anl_element_stress(self._h, _p(u), em, es, _p(sig) if sig is not None else None,
                                            _p(vm) if vm is not None else None, _stream()), "anl_element_stress")

    def sensitivity(self, U, coef, xphys, dxp, phi, p, emin, E0, out, dv=None):
        nrhs = len(coef)
        _chk(U, _F64, nrhs * self.ndof, "U")
        for t, n in ((xphys, "xphys"), (phi, "phi"), (out, "out")):
            _chk(t, _F32, self.ne, n)
        if dxp is not None:
            _chk(dxp, _F32, self.ne, "dxp")
        if dv is not None:
            _chk(dv, _F32, self.ne, "dv")
        c = (ctypes.c_double * nrhs)(*[float(v) for v in coef])
        N.check(self.lib.anl_sensitivity(self._h, _p(U), nrhs, c, _p(xphys),
                                         _p(dxp) if dxp is not None else None, _p(phi), float(p), float(emin),
                                         float(E0), _p(out), _p(dv) if dv is not None else None, _stream()),
                "anl_sensitivity")

    def stiffness_scale(self, xphys, phi, E0, emin, p, escale):
        for t, n in ((xphys, "xphys"), (phi, "phi"), (escale, "escale")):
            _chk(t, _F32, self.ne, n)
        N.check(self.lib.anl_stiffness_scale(self._h, _p(xphys), _p(phi), float(E0), float(emin), float(p),
                                             _p(escale), _stream()), "anl_stiffness_scale")

    # -- filter
    def filter_init(self, r):
        N.check(self.lib.anl_filter_init(self._h, float(r), _stream()), "anl_filter_init")
        self.filter_r = float(r)

    def filter_fwd(self, x, out):
        _chk(x, _F32, self.ne, "in")
        _chk(out, _F32, self.ne, "out")
        N.check(self.lib.anl_filter_fwd(self._h, _p(x), _p(out), _stream()), "anl_filter_fwd")

    def filter_bwd(self, x, out):
        _chk(x, _F32, self.ne, "in")
        _chk(out, _F32, self.ne, "out")
        N.check(self.lib.anl_filter_bwd(self._h, _p(x), _p(out), _stream()), "anl_filter_bwd")

    def physical(self, x, frozen, beta, eta, xphys, dxp=None):
        _chk(x, _F32, self.ne, "x")
        _chk(frozen, _U8, self.ne, "frozen")
        _chk(xphys, _F32, self.ne, "xphys")
        if dxp is not None:
            _chk(dxp, _F32, self.ne, "dxp")
        N.check(self.lib.anl_physical(self._h, _p(x), _p(frozen), float(beta), float(eta), _p(xphys),
                                      _p(dxp) if dxp is not None else None, _stream()), "anl_physical")

    # -- OC
    def oc_update(self, x, dcx, dvx, phi, frozen, move, beta, eta, vtarget, xnew):
        for t, n in ((x, "x"), (dcx, "dcx"), (dvx, "dvx"), (phi, "phi"), (xnew, "xnew")):
            _chk(t, _F32, self.ne, n)
        _chk(frozen, _U8, self.ne, "frozen")
        steps = ctypes.c_int(0)
        lam = ctypes.c_double(0.0)
        N.check(self.lib.anl_oc_update(self._h, _p(x), _p(dcx), _p(dvx), _p(phi), _p(frozen), float(move),
                                       float(beta), float(eta), float(vtarget), _p(xnew), ctypes.byref(steps),
                                       ctypes.byref(lam), _stream()), "anl_oc_update")
        return int(steps.value), float(lam.value)

    def design_stats(self, xold, xnew, xphys, phi, frozen):
        for t, n in ((xold, "xold"), (xnew, "xnew"), (xphys, "xphys"), (phi, "phi")):
            _chk(t, _F32, self.ne, n)
        _chk(frozen, _U8, self.ne, "frozen")
        out = (ctypes.c_double * 4)()
        N.check(self.lib.anl_design_stats(self._h, _p(xold), _p(xnew), _p(xphys), _p(phi), _p(frozen), out,
                                          _stream()), "anl_design_stats")
        return float(out[0]), float(out[1]), float(out[2]), int(out[3])


def to_dev(a, dtype):
    """numpy -> contiguous CUDA tensor of the given torch dtype."""
    return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype).contiguous()
