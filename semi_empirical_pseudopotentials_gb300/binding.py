"""ctypes binding of libsep_gb300.so (include/sep_gb300.h).

Arrays are numpy float64 / complex128 in the reference's layouts: grids x
fastest (filter/init.c:139-141), state blocks state-major
(psitot[state * ngrid + g], filter/main.c:86), complex interleaved.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsep_gb300.so")

PREC = {"f64": 0, "mixed": 1}

_lib = None
dp = C.POINTER(C.c_double)
lp = C.POINTER(C.c_long)
ip = C.POINTER(C.c_int)


class SepError(RuntimeError):
    """A non-zero status from the C ABI, with sep_last_error()'s message."""

    def __init__(self, status, msg):
        super().__init__(f"sep status {status}: {msg}")
        self.status = status


class Timing(C.Structure):
    _fields_ = [("energy_range_s", C.c_double), ("filter_s", C.c_double),
                ("ortho_s", C.c_double), ("rayleigh_ritz_s", C.c_double),
                ("sigma_s", C.c_double), ("total_s", C.c_double),
                ("power_iterations", C.c_long), ("mkept", C.c_long), ("h_applies", C.c_long),
                ("emax", C.c_double), ("dE", C.c_double), ("dt", C.c_double),
                ("polish_s", C.c_double)]


def lib():
    """Load the native library; raises if it was not built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise SepError(-5, f"{LIB_PATH} is missing: build it with "
                               "semi_empirical_pseudopotentials_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        L.sep_last_error.restype = C.c_char_p
        vp = C.c_void_p
        L.sep_ctx_create.argtypes = [lp, dp, C.c_double, dp, C.c_int, C.POINTER(vp)]
        for name in ("sep_ctx_destroy",):
            getattr(L, name).argtypes = [vp]
        L.sep_ctx_set_potential.argtypes = [vp, dp]
        L.sep_ctx_set_potential_dev.argtypes = [vp, vp]
        L.sep_ctx_info.argtypes = [vp, dp, dp, dp, lp]
        L.sep_ctx_stream.argtypes = [vp, C.POINTER(vp)]
        L.sep_ctx_set_graphs.argtypes = [vp, C.c_int]
        L.sep_ctx_set_block_steps.argtypes = [vp, C.c_int]
        L.sep_hamiltonian.argtypes = [vp, dp, dp, C.c_long]
        L.sep_hamiltonian_dev.argtypes = [vp, vp, vp, C.c_long]
        L.sep_hnorm.argtypes = [vp, dp, dp, C.c_long, C.c_double, C.c_double, C.c_double]
        L.sep_filter.argtypes = [vp, dp, C.c_long, dp, dp, C.c_long, C.c_long, C.c_double,
                                 C.c_double, dp]
        L.sep_filter_dev.argtypes = [vp, vp, C.c_long, dp, dp, C.c_long, C.c_long, C.c_double,
                                     C.c_double, vp]
        L.sep_normalize_all.argtypes = [vp, dp, C.c_long]
        L.sep_energy_all.argtypes = [vp, dp, C.c_long, dp]
        L.sep_energy_range.argtypes = [vp, C.c_double, dp, dp, lp]
        L.sep_ortho.argtypes = [vp, dp, C.c_long, lp]
        L.sep_rayleigh_ritz.argtypes = [vp, dp, C.c_long, dp]
        L.sep_sigma.argtypes = [vp, dp, C.c_long, dp]
        L.sep_pipeline.argtypes = [vp, dp, C.c_long, dp, C.c_long, C.c_long, C.c_double,
                                   C.c_double, dp, dp, dp, lp, C.POINTER(Timing)]
        L.sep_filter_chunk_plan.argtypes = [C.c_long, C.c_long, C.c_int, C.c_double, lp,
                                             C.c_long, lp]
        L.sep_coefficients.argtypes = [C.c_long, C.c_long, C.c_double, C.c_double, C.c_double,
                                       dp, dp, dp, dp]
        L.sep_start_states.argtypes = [C.c_long, C.c_long, C.c_long, C.c_double, dp]
        L.sep_ksqr.argtypes = [lp, dp, C.c_double, dp]
        L.sep_form_factor_table.argtypes = [dp, C.c_double, dp, dp]
        L.sep_vbuild.argtypes = [vp, C.c_long, dp, ip, dp, C.c_long, dp, dp, lp, C.c_long, dp,
                                 dp, C.c_int]
        L.sep_vbuild_backward.argtypes = [vp, C.c_long, dp, ip, dp, C.c_long, dp, dp, lp,
                                          C.c_long, dp, dp, dp, dp]
        L.sep_time_passes.argtypes = [vp, C.c_long, C.c_int, dp]
        L.sep_time_fused_step.argtypes = [vp, C.c_long, C.c_int, dp]
        L.sep_ctx_set_arith.argtypes = [vp, C.c_int]
        L.sep_hf_density.argtypes = [vp, dp, C.c_long, dp, dp]
        L.sep_ctx_autotune.argtypes = [vp, C.c_long, C.c_int, ip]
        L.sep_batch_create.argtypes = [C.c_int, C.POINTER(vp), lp, C.c_long, C.c_long,
                                       C.POINTER(vp)]
        L.sep_batch_io.argtypes = [vp, C.c_int, C.POINTER(vp), C.POINTER(vp)]
        L.sep_batch_set_coefficients.argtypes = [vp, C.c_int, dp, dp, C.c_double, C.c_double]
        L.sep_batch_run.argtypes = [vp]
        L.sep_batch_destroy.argtypes = [vp]
        L.sep_batch_load_start.argtypes = [vp, C.c_int, dp]
        L.sep_batch_read_out.argtypes = [vp, C.c_int, dp]
        L.sep_ctx_set_tiles.argtypes = [vp, ip]
        L.sep_form_factor_backward.argtypes = [dp, C.c_double, dp, dp]
        L.sep_ctx_set_subspace.argtypes = [vp, C.c_int]
        L.sep_ctx_set_fusion.argtypes = [vp, C.c_int]
        L.sep_ctx_set_refine.argtypes = [vp, C.c_int]
        L.sep_ctx_set_polish.argtypes = [vp, C.c_long, C.c_double]
        L.sep_ctx_set_eigensolver.argtypes = [vp, C.c_int]
        L.sep_subspace_gemm.argtypes = [vp, dp, dp, C.c_long, C.c_long, C.c_long, C.c_double,
                                        C.c_int, dp]
        L.sep_subspace_rotate.argtypes = [vp, dp, dp, C.c_long, C.c_long, C.c_long, dp]
        L.sep_subspace_gemm_dev.argtypes = [vp, vp, vp, C.c_long, C.c_long, C.c_long, C.c_double,
                                            C.c_int, vp]
        L.sep_potential_from_params.argtypes = [vp, C.c_long, dp, ip, dp, C.c_long, dp, C.c_double,
                                                dp, dp]
        L.sep_band_edge_backward.argtypes = [vp, C.c_long, dp, ip, dp, C.c_long, dp, C.c_double,
                                             dp, dp, C.c_long, dp, dp]
        cp = C.c_char_p
        L.sep_write_states.argtypes = [cp, dp, C.c_long, C.c_long]
        L.sep_write_eval.argtypes = [cp, dp, dp, C.c_long]
        L.sep_write_filter_eval.argtypes = [cp, dp, dp, C.c_long]
        L.sep_read_grid_source.argtypes = [cp, lp]
        L.sep_combine_outputs.argtypes = [C.c_int, C.POINTER(cp), cp, cp, C.c_long, cp, C.c_int,
                                          lp, lp]
        L.sep_bulk_basis.argtypes = [dp, C.c_double, C.c_long, lp, dp]
        L.sep_bulk_create.argtypes = [C.c_long, dp, C.c_long, dp, ip, C.c_long, C.c_long, dp,
                                      C.c_double, C.c_long, C.POINTER(vp)]
        L.sep_bulk_bands.argtypes = [vp, dp, dp]
        L.sep_bulk_bands_keep.argtypes = [vp, dp, dp]
        L.sep_bulk_bands_backward.argtypes = [vp, dp, dp, dp, dp]
        L.sep_bulk_solver_path.argtypes = [vp, ip]
        L.sep_bulk_set_solver.argtypes = [vp, C.c_int]
        L.sep_bulk_set_eigensolver.argtypes = [vp, C.c_int]
        L.sep_hermitian_lowest.argtypes = [dp, C.c_long, C.c_long, C.c_long, C.c_int, dp, dp]
        L.sep_bulk_destroy.argtypes = [vp]
        L.sep_spinor_vso.argtypes = [dp, C.c_long, C.c_long, C.c_long, vp, lp, C.c_double,
                                     C.c_double, C.c_int, dp, dp]
        L.sep_spinor_neighbour_lists.argtypes = [C.c_long, C.c_long, C.c_long, dp, dp, dp,
                                                 C.c_long, dp, dp, C.c_double, C.c_long, vp, lp]
        L.sep_spinor_vso_dev.argtypes = [vp, C.c_long, C.c_long, C.c_long, vp, vp, C.c_double,
                                         C.c_double, C.c_int, vp, vp, vp]
        _lib = L
    return _lib


def _check(status):
    if status != 0:
        raise SepError(status, lib().sep_last_error().decode(errors="replace"))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a):
    return a.ctypes.data_as(dp)


def device_count():
    n = C.c_int()
    _check(lib().sep_device_count(C.byref(n)))
    return n.value


def filter_chunk_plan(pairs, max_pairs, host_buffers=True, copy_ratio=-1.0):
    """Pair counts of the chunks sep_filter runs (see sep_filter_chunk_plan)."""
    counts = np.zeros(64, dtype=np.int64)
    nchunks = C.c_long(0)
    _check(lib().sep_filter_chunk_plan(int(pairs), int(max_pairs), 1 if host_buffers else 0,
                                       float(copy_ratio), counts.ctypes.data_as(lp), 64,
                                       C.byref(nchunks)))
    return [int(x) for x in counts[:nchunks.value]]


# ---- host helpers (bit-identical to the reference) --------------------------
def coefficients(el, nc, dE, vmin, dt):
    """filter/coeff.c:16-63 -> (an_re [ms, nc], an_im [ms, nc], zn [nc])."""
    el = _f64(el)
    ms = len(el)
    ar, ai, zn = np.empty((ms, nc)), np.empty((ms, nc)), np.empty(nc)
    _check(lib().sep_coefficients(ms, nc, dE, vmin, dt, _p(el), _p(ar), _p(ai), _p(zn)))
    return ar, ai, zn


def start_states(idum, ns, ngrid, dv):
    """filter/main.c:82-89 with init_psi (filter/init.c:236-251): [ns, ngrid]."""
    out = np.empty((ns, ngrid))
    _check(lib().sep_start_states(idum, ns, ngrid, dv, _p(out)))
    return out


def ksqr(dims, steps, ekinmax=10.0):
    dims_a = (C.c_long * 3)(*dims)
    steps_a = _f64(steps)
    out = np.empty(int(np.prod(dims)))
    _check(lib().sep_ksqr(dims_a, _p(steps_a), ekinmax, _p(out)))
    return out


def form_factor_table(params, vol_per_atom):
    """pseudopotFitting/pot.c:35-63 -> (r[1024], v[1024]) unshifted."""
    a = _f64(params)
    r, v = np.empty(1024), np.empty(1024)
    _check(lib().sep_form_factor_table(_p(a), vol_per_atom, _p(r), _p(v)))
    return r, v


def form_factor_backward(params, vol_per_atom, dtab):
    """dL/da0..a3 from dL/d(shifted 1024-point table), host only."""
    a, d = _f64(params), _f64(dtab)
    if d.shape != (1024,):
        raise ValueError("dtab must hold 1024 values")
    g = np.empty(4)
    _check(lib().sep_form_factor_backward(_p(a), vol_per_atom, _p(d), _p(g)))
    return g


def hermitian_lowest(a, nw, vectors=True):
    """The lowest nw eigenpairs of each Hermitian matrix a[m] (nmat x n x n,
    complex) with the library's batched solver: (w [nmat, nw], v [nmat, n,
    nw] or None), the columns of v unit eigenvectors."""
    a = np.asarray(a, dtype=np.complex128)
    if a.ndim == 2:
        a = a[None]
    nmat, n, n2 = a.shape
    if n != n2:
        raise ValueError("square matrices")
    # column-major per matrix: the transpose of each row-major matrix
    at = np.ascontiguousarray(np.transpose(a, (0, 2, 1)))
    w = np.empty((nmat, nw))
    v = np.empty((nmat, nw, n), dtype=np.complex128) if vectors else None
    _check(lib().sep_hermitian_lowest(at.view(np.float64).ctypes.data_as(dp), n, nmat, nw,
                                      1 if vectors else 0, _p(w),
                                      v.view(np.float64).ctypes.data_as(dp) if vectors else None))
    return w, (np.transpose(v, (0, 2, 1)) if vectors else None)


class Context:
    """One grid and one local potential on the GPU (sep_ctx)."""

    def __init__(self, dims, steps, potl=None, precision="f64", ekinmax=10.0):
        self.dims = tuple(int(d) for d in dims)
        self.ngrid = int(np.prod(self.dims))
        self.steps = tuple(float(s) for s in steps)
        self.precision = precision
        h = C.c_void_p()
        dims_a = (C.c_long * 3)(*self.dims)
        steps_a = _f64(self.steps)
        pot = None if potl is None else _f64(potl)
        _check(lib().sep_ctx_create(dims_a, _p(steps_a), ekinmax,
                                    None if pot is None else _p(pot), PREC[precision],
                                    C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.sep_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    # -- properties
    def info(self):
        vmin, vmax, dv, n = C.c_double(), C.c_double(), C.c_double(), C.c_long()
        _check(lib().sep_ctx_info(self.h, C.byref(vmin), C.byref(vmax), C.byref(dv),
                                  C.byref(n)))
        return {"vmin": vmin.value, "vmax": vmax.value, "dv": dv.value, "ngrid": n.value}

    @property
    def dv(self):
        return self.info()["dv"]

    def stream(self):
        s = C.c_void_p()
        _check(lib().sep_ctx_stream(self.h, C.byref(s)))
        return s.value

    def set_potential(self, potl):
        pot = _f64(potl)
        _check(lib().sep_ctx_set_potential(self.h, _p(pot)))

    def set_graphs(self, enable):
        _check(lib().sep_ctx_set_graphs(self.h, 1 if enable else 0))

    def set_block_steps(self, k):
        """Newton steps per accumulation pass, 1 <= k <= 128 (default 32); the
        history holds k grids per pair of states."""
        _check(lib().sep_ctx_set_block_steps(self.h, int(k)))

    # -- stages
    def hamiltonian(self, psi):
        """filter/hamiltonian.c:11-23 on complex grids [m, N] (or [N])."""
        z = np.ascontiguousarray(psi, dtype=np.complex128)
        shape = z.shape
        z = z.reshape(-1, self.ngrid)
        out = np.empty_like(z)
        _check(lib().sep_hamiltonian(self.h, z.ctypes.data_as(dp), out.ctypes.data_as(dp),
                                     z.shape[0]))
        return out.reshape(shape)

    def hnorm(self, psim1, dE_1, vmin, zm1):
        z = np.ascontiguousarray(psim1, dtype=np.complex128)
        shape = z.shape
        z = z.reshape(-1, self.ngrid)
        out = np.empty_like(z)
        _check(lib().sep_hnorm(self.h, z.ctypes.data_as(dp), out.ctypes.data_as(dp),
                               z.shape[0], dE_1, vmin, zm1))
        return out.reshape(shape)

    def filter(self, start, an_re, zn, dE_1, vmin, out=None):
        """filter/filter.c:59-83 for [ns, N] start states -> [ns, ms, N]."""
        start = _f64(start).reshape(-1, self.ngrid)
        an_re = _f64(an_re)
        ms, nc = an_re.shape
        zn = _f64(zn)
        if out is None:
            out = np.empty((start.shape[0], ms, self.ngrid))
        elif (out.dtype != np.float64 or not out.flags.c_contiguous or
              out.size != start.shape[0] * ms * self.ngrid):
            raise ValueError("out must be a C-contiguous float64 array of ns*ms*ngrid")
        _check(lib().sep_filter(self.h, _p(start), start.shape[0], _p(an_re), _p(zn), ms, nc,
                                dE_1, vmin, _p(out)))
        return out

    def filter_dev(self, start_ptr, ns, an_re, zn, dE_1, vmin, out_ptr):
        """Device-pointer variant (start: ns x N, out: ns x ms x N, float64)."""
        an_re = _f64(an_re)
        ms, nc = an_re.shape
        zn = _f64(zn)
        _check(lib().sep_filter_dev(self.h, C.c_void_p(start_ptr), ns, _p(an_re), _p(zn), ms,
                                    nc, dE_1, vmin, C.c_void_p(out_ptr)))

    def normalize_all(self, psi):
        psi = _f64(psi).copy()
        _check(lib().sep_normalize_all(self.h, _p(psi), psi.shape[0]))
        return psi

    def energy_all(self, psi):
        psi = _f64(psi)
        ene = np.empty(psi.shape[0])
        _check(lib().sep_energy_all(self.h, _p(psi), psi.shape[0], _p(ene)))
        return ene

    def energy_range(self, vmin):
        emax, dE, it = C.c_double(), C.c_double(), C.c_long()
        _check(lib().sep_energy_range(self.h, vmin, C.byref(emax), C.byref(dE), C.byref(it)))
        return emax.value, dE.value, it.value

    def ortho(self, psi):
        psi = _f64(psi).copy()
        k = C.c_long()
        _check(lib().sep_ortho(self.h, _p(psi), psi.shape[0], C.byref(k)))
        return psi[:k.value], k.value

    def rayleigh_ritz(self, psi):
        psi = _f64(psi).copy()
        ev = np.empty(psi.shape[0])
        _check(lib().sep_rayleigh_ritz(self.h, _p(psi), psi.shape[0], _p(ev)))
        return psi, ev

    def sigma(self, psi):
        psi = _f64(psi)
        s = np.empty(psi.shape[0])
        _check(lib().sep_sigma(self.h, _p(psi), psi.shape[0], _p(s)))
        return s

    def pipeline(self, start, el, nc, vmin, dE=0.0, want_psi=False):
        """filter/main.c:64-142 from given start states."""
        start = _f64(start).reshape(-1, self.ngrid)
        el = _f64(el)
        ns, ms = start.shape[0], len(el)
        m = ns * ms
        ev, sg = np.zeros(m), np.zeros(m)
        psi = np.empty((m, self.ngrid)) if want_psi else None
        k = C.c_long()
        t = Timing()
        _check(lib().sep_pipeline(self.h, _p(start), ns, _p(el), ms, nc, vmin, dE,
                                  None if psi is None else _p(psi), _p(ev), _p(sg),
                                  C.byref(k), C.byref(t)))
        kk = k.value
        return {"eval": ev[:kk], "sigma": sg[:kk], "mkept": kk,
                "psi": None if psi is None else psi[:kk],
                "timing": {f: getattr(t, f) for f, _ in Timing._fields_}}

    def hf_density(self, psi, w):
        """rho = dv sum_k w_k psi_k^2 (Hellmann-Feynman dL/dV for normalised states)."""
        psi = _f64(psi).reshape(-1, self.ngrid)
        w = _f64(w)
        rho = np.empty(self.ngrid)
        _check(lib().sep_hf_density(self.h, _p(psi), psi.shape[0], _p(w), _p(rho)))
        return rho

    def autotune(self, npairs, reps=5):
        """Pick the faster tile shape per Newton-step pass; returns the 5 picks."""
        ch = (C.c_int * 5)()
        _check(lib().sep_ctx_autotune(self.h, npairs, reps, ch))
        return list(ch)

    def set_tiles(self, choices):
        ch = (C.c_int * 5)(*[int(x) for x in choices])
        _check(lib().sep_ctx_set_tiles(self.h, ch))

    def time_passes(self, npairs, reps=10):
        """Average ms per launch: x fwd, y fwd, z fwd*k*inv, y inv, x inv+epi+fwd,
        accumulate, and the fused step's xy pass (plane or sub-plane form; 0
        when the context has no fused step)."""
        out = np.zeros(7)
        _check(lib().sep_time_passes(self.h, npairs, reps, _p(out)))
        return out

    def time_fused_step(self, npairs, reps=10):
        """Average ms per launch of the fused complex64 step's xy pass and z pass
        (plane form: xy plane pass and z line pass; sub-plane form: sub-plane
        pass and zy pass); zeros when the context has no fused step."""
        out = np.zeros(2)
        _check(lib().sep_time_fused_step(self.h, npairs, reps, _p(out)))
        return out

    def vbuild(self, xyz, types, tab_r, tab_v, tab_n, mins, scale=None, install=True):
        """filter/init.c:157-182 on this grid; tables [ntype, stride] (shifted)."""
        xyz = _f64(xyz)
        types = np.ascontiguousarray(types, dtype=np.int32)
        tab_r, tab_v = _f64(tab_r), _f64(tab_v)
        tab_n = np.ascontiguousarray(tab_n, dtype=np.int64)
        sc = None if scale is None else _f64(scale)
        mins = _f64(mins)
        out = np.empty(self.ngrid)
        _check(lib().sep_vbuild(self.h, len(xyz), _p(xyz), types.ctypes.data_as(ip),
                                None if sc is None else _p(sc), tab_r.shape[0], _p(tab_r),
                                _p(tab_v), tab_n.ctypes.data_as(lp), tab_r.shape[1], _p(mins),
                                _p(out), 1 if install else 0))
        return out

    def set_refine(self, steps):
        """FP64 residual-subspace steps after Rayleigh-Ritz in pipeline() (0..8)."""
        _check(lib().sep_ctx_set_refine(self.h, int(steps)))

    def set_polish(self, nc, guard=0.01):
        """FP64 polish of the window's Ritz pairs in pipeline(): nc Newton steps of
        one wide Gaussian at the window centre (0 = off), guard in hartree."""
        _check(lib().sep_ctx_set_polish(self.h, int(nc), float(guard)))

    def set_eigensolver(self, mode):
        """Dense symmetric eigensolves of ortho and Rayleigh-Ritz: the library's
        own solver ("native" or 1) or cuSOLVER ("cusolver" or 0)."""
        m = {"native": 1, "cusolver": 0}.get(mode, mode)
        _check(lib().sep_ctx_set_eigensolver(self.h, int(m)))

    def set_fusion(self, enable):
        """Fused two-pass complex64 Newton steps: the sub-plane and zy passes for
        cubic grids with nx in {96, 112, 128, 160, 192, 256}, else the xy plane
        pass for nx = ny in {40, 48, ..., 128}.  On by default; off: the four
        line passes."""
        _check(lib().sep_ctx_set_fusion(self.h, 1 if enable else 0))

    def set_arith(self, mode):
        """Arithmetic of the pipeline's FP64-class H applies (Rayleigh-Ritz, sigma,
        refinement, polish filter): "f64" (IEEE FP64) or "dd" (double-float on
        the FP32 pipe, about 48 significant bits; default for complex64
        contexts)."""
        _check(lib().sep_ctx_set_arith(self.h, {"f64": 0, "dd": 1}[mode]))

    def set_subspace(self, mode):
        """Subspace contractions on the tensor cores ("tc", default) or the FP64 pipe ("f64")."""
        _check(lib().sep_ctx_set_subspace(self.h, {"f64": 0, "tc": 1}[mode]))

    def subspace_gemm(self, A, B=None, alpha=1.0):
        """alpha A B^T through the context's subspace contraction (B None: A A^T)."""
        A = _f64(A)
        sym = B is None
        Bm = A if sym else _f64(B)
        if Bm.shape[1] != A.shape[1]:
            raise ValueError("A and B need the same number of columns")
        out = np.empty((A.shape[0], Bm.shape[0]))
        _check(lib().sep_subspace_gemm(self.h, _p(A), None if sym else _p(Bm), A.shape[0],
                                       Bm.shape[0], A.shape[1], alpha, 1 if sym else 0, _p(out)))
        return out

    def subspace_gemm_dev(self, A_ptr, B_ptr, m, n, k, C_ptr, alpha=1.0, sym=False):
        """Device-pointer form on the context's stream."""
        _check(lib().sep_subspace_gemm_dev(self.h, A_ptr, B_ptr, m, n, k, alpha, 1 if sym else 0,
                                           C_ptr))

    def subspace_rotate(self, W, X):
        """W X through the context's subspace contraction."""
        W, X = _f64(W), _f64(X)
        if W.shape[1] != X.shape[0]:
            raise ValueError("inner dimensions differ")
        out = np.empty((W.shape[0], X.shape[1]))
        _check(lib().sep_subspace_rotate(self.h, _p(W), _p(X), W.shape[0], W.shape[1],
                                         X.shape[1], _p(out)))
        return out

    def potential_from_params(self, xyz, types, params, vol_per_atom, mins, scale=None):
        """Shifted form-factor tables of theta (ntype x 4), then V(r), installed."""
        xyz, th, mins = _f64(xyz), _f64(params).reshape(-1, 4), _f64(mins)
        types = np.ascontiguousarray(types, dtype=np.int32)
        sc = None if scale is None else _f64(scale)
        out = np.empty(self.ngrid)
        _check(lib().sep_potential_from_params(self.h, len(xyz), _p(xyz), types.ctypes.data_as(ip),
                                               None if sc is None else _p(sc), th.shape[0],
                                               _p(th), vol_per_atom, _p(mins), _p(out)))
        return out

    def band_edge_backward(self, xyz, types, params, vol_per_atom, mins, psi, dL_dE, scale=None):
        """dL/dtheta (ntype x 4) for Ritz states psi (m x ngrid) and dL/dE (m)."""
        xyz, th, mins = _f64(xyz), _f64(params).reshape(-1, 4), _f64(mins)
        types = np.ascontiguousarray(types, dtype=np.int32)
        sc = None if scale is None else _f64(scale)
        psi = _f64(psi).reshape(-1, self.ngrid)
        w = _f64(dL_dE)
        if len(w) != psi.shape[0]:
            raise ValueError("one dL/dE per state")
        g = np.empty_like(th)
        _check(lib().sep_band_edge_backward(self.h, len(xyz), _p(xyz), types.ctypes.data_as(ip),
                                            None if sc is None else _p(sc), th.shape[0], _p(th),
                                            vol_per_atom, _p(mins), _p(psi), psi.shape[0], _p(w),
                                            _p(g)))
        return g

    def vbuild_backward(self, xyz, types, tab_r, tab_v, tab_n, mins, dpotl, scale=None):
        xyz = _f64(xyz)
        types = np.ascontiguousarray(types, dtype=np.int32)
        tab_r, tab_v = _f64(tab_r), _f64(tab_v)
        tab_n = np.ascontiguousarray(tab_n, dtype=np.int64)
        sc = None if scale is None else _f64(scale)
        mins = _f64(mins)
        g = _f64(dpotl)
        dtab = np.zeros_like(tab_v)
        dsc = None if sc is None else np.zeros(len(xyz))
        _check(lib().sep_vbuild_backward(self.h, len(xyz), _p(xyz), types.ctypes.data_as(ip),
                                         None if sc is None else _p(sc), tab_r.shape[0],
                                         _p(tab_r), _p(tab_v), tab_n.ctypes.data_as(lp),
                                         tab_r.shape[1], _p(mins), _p(g), _p(dtab),
                                         None if dsc is None else _p(dsc)))
        return dtab, dsc


class Batch:
    """Several nanocrystals (one Context each, grids may differ) filtered by a
    single CUDA graph launch (sep_batch_*)."""

    def __init__(self, contexts, ns, ms, nc):
        self.contexts = list(contexts)
        arr = (C.c_void_p * len(self.contexts))(*[c.h.value for c in self.contexts])
        nsa = (C.c_long * len(self.contexts))(*[int(x) for x in ns])
        h = C.c_void_p()
        _check(lib().sep_batch_create(len(self.contexts), arr, nsa, ms, nc, C.byref(h)))
        self.h = h
        self.ns = [int(x) for x in ns]
        self.ms, self.nc = ms, nc

    def io(self, job):
        s, o = C.c_void_p(), C.c_void_p()
        _check(lib().sep_batch_io(self.h, job, C.byref(s), C.byref(o)))
        return s.value, o.value

    def set_coefficients(self, job, an_re, zn, dE_1, vmin):
        an_re, zn = _f64(an_re), _f64(zn)
        _check(lib().sep_batch_set_coefficients(self.h, job, _p(an_re), _p(zn), dE_1, vmin))

    def load_start(self, job, start):
        start = _f64(start)
        if start.size != self.ns[job] * self.contexts[job].ngrid:
            raise ValueError("start must hold ns x ngrid values")
        _check(lib().sep_batch_load_start(self.h, job, _p(start)))

    def read_out(self, job):
        out = np.empty((self.ns[job], self.ms, self.contexts[job].ngrid))
        _check(lib().sep_batch_read_out(self.h, job, _p(out)))
        return out

    def run(self):
        _check(lib().sep_batch_run(self.h))

    def close(self):
        if getattr(self, "h", None) and self.h.value and _lib is not None:
            _lib.sep_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
