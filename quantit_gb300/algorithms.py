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
    """dmrg_logger (include/dmrg_logger.h:27-99): ``init`` before the first sweep,
    ``it_log_all`` after every sweep and ``end_log_all`` once when the driver stops;
    both default to ``log_all`` = ``log_step`` + ``log_energy`` + ``log_bond_dims``.
    ``log_truncation`` (no reference counterpart) receives, before each
    ``it_log_all``, the sweep's largest relative discarded weight (sum of dropped
    s^2 over sum of all s^2 of a bond's truncation)."""

    def log_step(self, step):
        pass

    def log_energy(self, energy):
        pass

    def log_bond_dims(self, mps):
        pass

    def log_truncation(self, weight):
        pass

    def init(self, options):
        pass

    def it_log_all(self, step, energy, mps):
        self.log_all(step, energy, mps)

    def end_log_all(self, step, energy, mps):
        self.log_all(step, energy, mps)

    def log_all(self, step, energy, mps):
        self.log_step(step)
        self.log_energy(energy)
        self.log_bond_dims(mps)


dmrg_default_logger = dmrg_logger


def _middle_bond_dim(mps):
    """max of the first and last leg sizes of the middle site (dmrg_logger.h:122-126)."""
    sizes = mps[len(mps) // 2].sizes()
    return int(max(sizes[0], sizes[2]))


class dmrg_log_simple(dmrg_logger):
    """dmrg_log_simple (dmrg_logger.h:109-132): the step and the middle bond dimension,
    recorded from log_all (its it_log_all does nothing, as in the reference)."""

    def __init__(self):
        self.it_num = 0
        self.middle_bond_dim = 0

    def log_step(self, step):
        self.it_num = step

    def log_bond_dims(self, mps):
        self.middle_bond_dim = _middle_bond_dim(mps)

    def it_log_all(self, step, energy, mps):
        pass


class dmrg_log_sweeptime(dmrg_logger):
    """dmrg_log_sweeptime (dmrg_logger.h:133-185): per sweep, the wall time since the
    previous call (time_list), the middle bond dimension (bond_list), the energy and
    the sweep's largest relative discarded weight."""

    def __init__(self):
        import time
        self._clock = time.perf_counter
        self.it_num = 0
        self.middle_bond_dim = 0
        self.time_list, self.bond_list = [], []
        self.energies, self.truncated_weights = [], []
        self._then = self._clock()
        self._pending_trunc = None

    @property
    def times(self):
        return self.time_list

    def init(self, options):
        self._then = self._clock()
        self.time_list, self.bond_list, self.energies, self.truncated_weights = [], [], [], []

    def log_step(self, step):
        self.it_num = step

    def log_energy(self, energy):
        self.energies.append(energy)

    def log_bond_dims(self, mps):
        self.middle_bond_dim = _middle_bond_dim(mps)

    def log_truncation(self, weight):
        self._pending_trunc = weight

    def it_log_all(self, step, energy, mps):
        now = self._clock()
        self.time_list.append(now - self._then)
        self._then = now
        self.log_bond_dims(mps)
        self.bond_list.append(self.middle_bond_dim)
        self.truncated_weights.append(self._pending_trunc)
        self.log_step(step)
        self.log_energy(energy)

    def end_log_all(self, step, energy, mps):
        pass


def _borrowed_mps(n, handles, oc):
    """Owned copies (shared device data) of the state handles a callback receives."""
    from .networks import bMPS
    out = []
    for i in range(n):
        h = C.c_void_p()
        _lib.call("qtt_bt_clone", C.c_void_p(handles[i]), C.byref(h))
        out.append(btensor._wrap(h))
    return bMPS(out, int(oc))


def dmrg(mpo, mps, options=None, logger=None):
    """dmrg(bMPO, bMPS, dmrg_options, logger): optimises ``mps`` in place (its tensors
    are replaced and its orthogonality_center updated); returns the energy.  An
    exception raised by the logger is re-raised when the driver returns."""
    options = options or dmrg_options()
    L = len(mpo)
    if len(mps) != L:
        raise ValueError("MPO and MPS lengths differ")
    mpo_h = (C.c_void_p * L)(*[t._h.value for t in mpo])
    mps_h = (C.c_void_p * L)(*[t._h.value for t in mps])
    oc = C.c_int64(int(getattr(mps, "orthogonality_center", 0)))
    E = C.c_double()
    opt = options._c()
    lg = None
    errors = []
    if logger is not None:
        def guard(f):
            def run(*a):
                try:
                    f(*a)
                except BaseException as e:  # re-raised after the driver returns
                    errors.append(e)
            return run

        def on_init(user, o):
            logger.init(options)

        def on_it(user, step, e, secs, trunc, n, hs, c):
            logger.log_truncation(float(trunc))
            logger.it_log_all(int(step), float(e), _borrowed_mps(n, hs, c))

        def on_end(user, step, e, n, hs, c):
            logger.end_log_all(int(step), float(e), _borrowed_mps(n, hs, c))
        lg = _lib.DmrgLoggerC(None, _lib.LOG_INIT(guard(on_init)), _lib.LOG_IT(guard(on_it)),
                              _lib.LOG_END(guard(on_end)))
    _lib.call("qtt_dmrg_logged", L, mpo_h, mps_h, C.byref(oc), C.byref(opt), C.byref(lg) if lg else None,
              C.byref(E))
    for i in range(L):
        mps[i] = btensor._wrap(C.c_void_p(mps_h[i]))
    if hasattr(mps, "orthogonality_center"):
        mps.orthogonality_center = oc.value
    if errors:
        raise errors[0]
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


def trivial_edge(state, state_leg, mpo, mpo_leg):
    """The all-ones edge environment (generate_env_impl, sources/dmrg.cpp:371-391):
    trivial_edge(mps[0], 0, mpo[0], 0) on the left, (mps[-1], 2, mpo[-1], 2) on the right."""
    h = C.c_void_p()
    _lib.call("qtt_trivial_edge", state._h, int(state_leg), mpo._h, int(mpo_leg), C.byref(h))
    return btensor._wrap(h)


def environments(mpo, mps, bonds):
    """{bond b: (L, R)}: the left environment of sites 0..b-1 and the right environment
    of sites b+2..L-1 of the two-site update at bond b (generate_env_impl,
    sources/dmrg.cpp:371-409), contracted on the GPU from the edges inward."""
    L = len(mps)
    want = sorted(set(int(b) for b in bonds))
    if not want or want[0] < 0 or want[-1] > L - 2:
        raise ValueError("bond index out of range")
    left, right = {}, {}
    env = trivial_edge(mps[0], 0, mpo[0], 0)
    for i in range(want[-1] + 1):
        if i in want:
            left[i] = env
        env = compute_left_env(mpo[i], mps[i], env)
    env = trivial_edge(mps[L - 1], 2, mpo[L - 1], 2)
    if L - 2 in want:
        right[L - 2] = env
    for i in range(L - 1, want[0] + 1, -1):
        env = compute_right_env(mpo[i], mps[i], env)
        if i - 2 in want:
            right[i - 2] = env
    return {b: (left[b], right[b]) for b in want}


def compute_right_env(W, A, R):
    h = C.c_void_p()
    _lib.call("qtt_compute_right_env", W._h, A._h, R._h, C.byref(h))
    return btensor._wrap(h)
