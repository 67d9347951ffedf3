"""Two-site DMRG, mirroring ``quantit.algorithms`` (python_binding/algorithm.cpp:17-194)."""
import ctypes as C

from . import _lib
from .tensor import btensor

SIZE_MAX = 2 ** 63 - 1
GEMM_MODES = {"f64": 0, "tf32x3": 1, "bf16x3": 2}


class dmrg_options:
    """dmrg_options (include/dmrg_options.h:15-58) plus the block-GEMM precision."""

    def __init__(self, *, cutoff=1e-6, convergence_criterion=1e-5, max_bond=SIZE_MAX, min_bond=4,
                 maximum_iterations=1000, gemm="f64", final_energy_fp64=True, lanczos_steps=1,
                 cuda_graphs=True, svd_warm_start=True):
        self.cutoff = cutoff
        self.convergence_criterion = convergence_criterion
        self.maximum_bond = max_bond
        self.minimum_bond = min_bond
        self.maximum_iterations = maximum_iterations
        self.gemm = gemm
        # mixed precision: the FP64 <psi|H|psi>/<psi|psi> of the state replaces the Ritz
        # value after every sweep (convergence test, log) and as the returned energy
        self.final_energy_fp64 = final_energy_fp64
        # 1: QuantiT's one-step update; k > 1: k-step Lanczos per bond
        self.lanczos_steps = lanczos_steps
        # k-step Lanczos: replay each bond's matvec from a captured CUDA graph
        self.cuda_graphs = cuda_graphs
        # start each bond's sector SVD from that bond's previous rotation (exact either way)
        self.svd_warm_start = svd_warm_start

    def _c(self):
        o = _lib.DmrgOptionsC()
        o.cutoff = float(self.cutoff)
        o.convergence_criterion = float(self.convergence_criterion)
        o.maximum_bond = int(min(self.maximum_bond, SIZE_MAX))
        o.minimum_bond = int(self.minimum_bond)
        o.maximum_iterations = int(self.maximum_iterations)
        o.gemm_mode = GEMM_MODES[self.gemm] if isinstance(self.gemm, str) else int(self.gemm)
        o.final_energy_fp64 = int(bool(self.final_energy_fp64))
        o.lanczos_steps = int(self.lanczos_steps)
        o.cuda_graphs = int(bool(self.cuda_graphs))
        o.svd_warm_start = int(bool(self.svd_warm_start))
        return o


class dmrg_logger:
    """Per-sweep callback (dmrg_logger::it_log_all, include/dmrg_logger.h:53)."""

    def it_log_all(self, sweep, energy, seconds):
        pass


class dmrg_log_sweeptime(dmrg_logger):
    """Records every sweep's energy and wall time (dmrg_log_sweeptime, dmrg_logger.h:133-185)."""

    def __init__(self):
        self.energies = []
        self.times = []

    def it_log_all(self, sweep, energy, seconds):
        self.energies.append(energy)
        self.times.append(seconds)


def dmrg(mpo, mps, options=None, logger=None):
    """dmrg(bMPO, bMPS, dmrg_options, logger): optimises ``mps`` in place (its tensors
    are replaced and its orthogonality_center updated); returns the energy."""
    options = options or dmrg_options()
    L = len(mpo)
    if len(mps) != L:
        raise ValueError("MPO and MPS lengths differ")
    mpo_h = (C.c_void_p * L)(*[t._h.value for t in mpo])
    mps_h = (C.c_void_p * L)(*[t._h.value for t in mps])
    oc = C.c_int64(int(getattr(mps, "orthogonality_center", 0)))
    E = C.c_double()
    opt = options._c()
    cb = _lib.LOG_FN(lambda user, it, e, s: logger.it_log_all(int(it), float(e), float(s))) if logger else None
    _lib.call("qtt_dmrg", L, mpo_h, mps_h, C.byref(oc), C.byref(opt), C.cast(cb, C.c_void_p) if cb else None,
              None, C.byref(E))
    for i in range(L):
        mps[i] = btensor._wrap(C.c_void_p(mps_h[i]))
    if hasattr(mps, "orthogonality_center"):
        mps.orthogonality_center = oc.value
    return E.value


def mps_energy(mpo, mps):
    """(<psi|H|psi>, <psi|psi>) contracted in FP64 (contract(bMPS, bMPS, bMPO))."""
    L = len(mpo)
    mpo_h = (C.c_void_p * L)(*[t._h.value for t in mpo])
    mps_h = (C.c_void_p * L)(*[t._h.value for t in mps])
    e, n = C.c_double(), C.c_double()
    _lib.call("qtt_mps_energy", L, mpo_h, mps_h, C.byref(e), C.byref(n))
    return e.value, n.value


def hamil2site_times_state(state, hamil, Lenv, Renv):
    h = C.c_void_p()
    _lib.call("qtt_hamil2site_times_state", state._h, hamil._h, Lenv._h, Renv._h, C.byref(h))
    return btensor._wrap(h)


def one_step_lanczos(state, hamil, Lenv, Renv):
    psi, a0, a1, b = C.c_void_p(), C.c_double(), C.c_double(), C.c_double()
    _lib.call("qtt_one_step_lanczos", state._h, hamil._h, Lenv._h, Renv._h, C.byref(psi), C.byref(a0), C.byref(a1),
              C.byref(b))
    return btensor._wrap(psi), a0.value, a1.value, b.value


def eig2x2(a0, a1, b):
    E, o, n = C.c_double(), C.c_double(), C.c_double()
    _lib.call("qtt_eig2x2", float(a0), float(a1), float(b), C.byref(E), C.byref(o), C.byref(n))
    return E.value, o.value, n.value


def compute_2sites_hamil(wl, wr):
    h = C.c_void_p()
    _lib.call("qtt_compute_2sites_hamil", wl._h, wr._h, C.byref(h))
    return btensor._wrap(h)


def compute_left_env(W, A, L):
    h = C.c_void_p()
    _lib.call("qtt_compute_left_env", W._h, A._h, L._h, C.byref(h))
    return btensor._wrap(h)


def compute_right_env(W, A, R):
    h = C.c_void_p()
    _lib.call("qtt_compute_right_env", W._h, A._h, R._h, C.byref(h))
    return btensor._wrap(h)
