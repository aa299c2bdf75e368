"""Python host mirror of the reference's NRG API over the C ABI (libnrggpu.so).

Names and argument meaning follow the reference:
  NrgCore          nrgcore<Imp,Bath>                   nrgcore/nrgcore.hpp:25-551
  update_system_operator                               nrgcore/sysOperator.hpp:36-133
  NrgData          NrgData (device-resident snapshots)  nrgcore/nrgData.hpp:31-302
  FdmSpectrum      fdmSpectrum<N>                        dynamics/fdmSpectrum.hpp:24-364
  FdmThermodynamics fdmThermodynamics<N>                 static/fdmThermodynamics.hpp:16-260
Errors raise RuntimeError like the reference's std::runtime_error.  There is
no CPU fallback: without the library or a CUDA device every call raises.
"""
import ctypes as C
import os
import weakref

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# NRG_GPU_LIB: path of another build of the library (A/B timing of two builds)
_LIBPATH = os.environ.get("NRG_GPU_LIB") or os.path.join(_HERE, "libnrggpu.so")
_lib = None

PREC_FP64, PREC_MIXED = 0, 1
FDM_POINTS = 100000


class NrgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("nrg error %d: %s" % (code, msg))
        self.code = code


class _EngineOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("precision", C.c_int), ("hbm_budget_bytes", C.c_uint64),
                ("verbose", C.c_int)]


class _SiteDesc(C.Structure):
    _fields_ = [("nq", C.c_int), ("nsect", C.c_int), ("qnum", C.POINTER(C.c_int)),
                ("dims", C.POINTER(C.c_int)), ("energies", C.POINTER(C.c_double)),
                ("chi", C.POINTER(C.c_double)), ("nops", C.c_int), ("nblk", C.c_int),
                ("blk_op", C.POINTER(C.c_int)), ("blk_row", C.POINTER(C.c_int)),
                ("blk_col", C.POINTER(C.c_int)), ("blk_data", C.POINTER(C.c_double))]


class _OpDesc(C.Structure):
    _fields_ = [("nops", C.c_int), ("nblk", C.c_int), ("blk_op", C.POINTER(C.c_int)),
                ("blk_row", C.POINTER(C.c_int)), ("blk_col", C.POINTER(C.c_int)),
                ("blk_rows", C.POINTER(C.c_int)), ("blk_cols", C.POINTER(C.c_int)),
                ("blk_data", C.POINTER(C.c_double))]


class RunInfo(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "iteration", "iteration_min", "n_pre_sectors", "n_cur_sectors", "n_all", "n_kept",
        "n_relgs", "nq", "n_device_blocks", "max_block", "n_snapshots", "device_bytes")]


EXPORTS = [
    "nrg_last_error", "nrg_engine_create", "nrg_engine_destroy", "nrg_engine_phase_times",
    "nrg_engine_launch_count", "nrg_engine_get_opts", "nrg_engine_fallback_count", "nrg_engine_memory",
    "nrg_engine_set_profiling", "nrg_engine_kernel_times", "nrg_engine_work_counters",
    "nrg_engine_set_autotune", "nrg_engine_autotune_report", "nrg_engine_set_eig_cluster",
    "nrg_engine_sync", "nrg_run_create", "nrg_run_destroy",
    "nrg_run_set_parameters", "nrg_run_set_bath", "nrg_run_add_site", "nrg_run_update_state",
    "nrg_run_check_discarded", "nrg_run_get_info", "nrg_run_get_all_eigenvalues",
    "nrg_run_get_relgs", "nrg_run_get_sectors", "nrg_run_get_eigenvalues_q", "nrg_run_get_kept",
    "nrg_run_get_coupled", "nrg_run_get_eigenvectors", "nrg_run_get_fdag_block",
    "nrg_opset_create", "nrg_opset_destroy", "nrg_opset_update", "nrg_opset_update_batch", "nrg_opset_get_block",
    "nrg_run_snapshot", "nrg_run_load_snapshot", "nrg_run_export_snapshots",
    "nrg_opset_list_blocks", "nrg_run_list_fdag_blocks", "nrg_run_list_snapshot_ops",
    "nrg_run_get_snapshot_op_block", "nrg_fdm_create", "nrg_fdm_destroy",
    "nrg_fdm_calc", "nrg_fdm_calc_batch", "nrg_fdm_get", "nrg_broaden", "nrg_thermo_create", "nrg_thermo_destroy",
    "nrg_thermo_calc", "nrg_thermo_final", "nrg_thermo_set_operator", "nrg_thermo_get_operator",
    "nrg_fdm_set_temperature", "nrg_fdm_get_static", "nrg_batch_add_site", "nrg_batch_update_state",
    "nrg_eigh_batched", "nrg_dgemm_tc", "nrg_broaden_noalloc",
    "nrg_server_create", "nrg_server_destroy", "nrg_server_submit", "nrg_server_wait",
    "nrg_server_result_info", "nrg_server_get_result", "nrg_server_release", "nrg_server_stats",
]
BROADEN_NOALLOC_MAX_BINS = 131072  # NRG_BROADEN_NOALLOC_MAX_BINS


def lib():
    """Load libnrggpu.so (built in-tree by nrgplusplus_gb300.build).  Raises if
    it is missing: the engine has no CPU fallback."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIBPATH):
            raise NrgError(6, "libnrggpu.so not built (run nrgplusplus_gb300.build)")
        L = C.CDLL(_LIBPATH)
        L.nrg_last_error.restype = C.c_char_p
        for name in EXPORTS:
            getattr(L, name)
        _lib = L
    return _lib


def _call(fn, *args):
    rc = fn(*args)
    if rc != 0:
        raise NrgError(rc, lib().nrg_last_error().decode())


C_double = C.c_double


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


class _SiteBuffers:
    """Keeps the numpy arrays behind one nrg_site_desc alive."""

    def __init__(self, site, need_chi):
        self.q = np.ascontiguousarray(np.array(site.qnums, dtype=np.int32).reshape(len(site.qnums), -1))
        self.dims = np.array([len(e) for e in site.energies], dtype=np.int32)
        self.E = np.ascontiguousarray(np.concatenate([np.asarray(e, float) for e in site.energies]))
        self.chi = np.ascontiguousarray(np.asarray(site.chi, float)) if need_chi else None
        ops, rows, cols, data = [], [], [], []
        for ip, d in enumerate(site.fdag):
            for (i, j), m in sorted(d.items()):
                ops.append(ip)
                rows.append(i)
                cols.append(j)
                data.append(np.ascontiguousarray(m, float).ravel())
        self.op = np.array(ops, dtype=np.int32)
        self.row = np.array(rows, dtype=np.int32)
        self.col = np.array(cols, dtype=np.int32)
        self.data = np.ascontiguousarray(np.concatenate(data) if data else np.zeros(1))
        self.desc = _SiteDesc(self.q.shape[1], len(self.dims), _ip(self.q), _ip(self.dims), _dp(self.E),
                              _dp(self.chi) if self.chi is not None else None, len(site.fdag),
                              len(self.op), _ip(self.op), _ip(self.row), _ip(self.col), _dp(self.data))


class Engine:
    """One GPU engine: device context, stream and allocator (nrg_engine)."""

    def __init__(self, precision=PREC_FP64, device=0, hbm_budget_bytes=0):
        self.h = C.c_void_p()
        self._children = weakref.WeakSet()
        opts = _EngineOpts(device, precision, hbm_budget_bytes, 0)
        _call(lib().nrg_engine_create, C.byref(opts), C.byref(self.h))
        self.precision = precision

    def _adopt(self, obj):
        self._children.add(obj)

    def close(self):
        """Release every object still open on this engine, then the engine."""
        if self.h:
            for ch in list(self._children):
                if not isinstance(ch, NrgCore):
                    ch.close()
            for ch in list(self._children):
                ch.close()
            lib().nrg_engine_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def phase_times(self):
        out = (C.c_double * 8)()
        n = C.c_int()
        _call(lib().nrg_engine_phase_times, self.h, out, 8, C.byref(n))
        return list(out)[:n.value]

    def launch_count(self):
        v = C.c_uint64()
        _call(lib().nrg_engine_launch_count, self.h, C.byref(v))
        return v.value

    def memory(self, reset_peak=False):
        """(device bytes held now, high-water mark) of this engine."""
        u, p = C.c_uint64(), C.c_uint64()
        _call(lib().nrg_engine_memory, self.h, C.byref(u), C.byref(p), int(reset_peak))
        return u.value, p.value

    def fallback_count(self):
        """Blocks of the mixed path re-solved in FP64 so far."""
        v = C.c_uint64()
        _call(lib().nrg_engine_fallback_count, self.h, C.byref(v))
        return v.value

    def set_autotune(self, on=True):
        """Launch-shape autotuner on / off (nrg_engine_set_autotune)."""
        _call(lib().nrg_engine_set_autotune, self.h, 1 if on else 0)

    def set_eig_cluster(self, mode):
        """Cluster eigensolver for blocks above one SM's shared memory:
        0 off, 1 when the launch's clusters fit one wave (default), 2 always
        (nrg_engine_set_eig_cluster)."""
        _call(lib().nrg_engine_set_eig_cluster, self.h, int(mode))

    def autotune_report(self):
        """The autotuner's decisions: one line per block-size histogram."""
        n = C.c_uint64()
        _call(lib().nrg_engine_autotune_report, self.h, None, C.c_uint64(0), C.byref(n))
        buf = C.create_string_buffer(n.value + 1)
        _call(lib().nrg_engine_autotune_report, self.h, buf, C.c_uint64(n.value + 1), C.byref(n))
        return [x for x in buf.value.decode().split("\n") if x]

    def work_counters(self, reset=False):
        """Algorithmic work since the last reset: {'F_eig', 'F_rot',
        'tc_useful', 'tc_bf16'} in flops (nrg_engine_work_counters)."""
        out = (C.c_double * 4)()
        n = C.c_int()
        _call(lib().nrg_engine_work_counters, self.h, out, 4, C.byref(n), int(reset))
        return dict(zip(("F_eig", "F_rot", "tc_useful", "tc_bf16"), list(out)[:n.value]))

    def sync(self):
        _call(lib().nrg_engine_sync, self.h)

    def set_profiling(self, on=True):
        _call(lib().nrg_engine_set_profiling, self.h, 1 if on else 0)

    def kernel_times(self):
        """{kernel: (ms, algorithmic flops or bytes, launches)} recorded since the last call."""
        cap = 64
        names = C.create_string_buffer(8192)
        ms = (C.c_double * cap)()
        work = (C.c_double * cap)()
        cnt = (C.c_uint64 * cap)()
        nk = C.c_int()
        _call(lib().nrg_engine_kernel_times, self.h, names, C.c_uint64(8192), ms, work, cnt, cap,
              C.byref(nk))
        keys = names.value.decode().split("\n")[:nk.value]
        return {k: (ms[i], work[i], cnt[i]) for i, k in enumerate(keys)}

    def eigh_batched(self, mats):
        """Eigen-decompose a list of dense symmetric blocks on the GPU
        (qmatrix::diag semantics): [(eigenvalues ascending, eigenvectors as columns)]."""
        dims = np.array([m.shape[0] for m in mats], dtype=np.int32)
        H = np.ascontiguousarray(np.concatenate([np.ascontiguousarray(m, float).ravel() for m in mats]))
        E = np.zeros(int(dims.sum()))
        U = np.zeros(H.size)
        _call(lib().nrg_eigh_batched, self.h, len(mats), _ip(dims), _dp(H), _dp(E), _dp(U))
        out, eo, uo = [], 0, 0
        for n in dims:
            n = int(n)
            out.append((E[eo:eo + n].copy(), U[uo:uo + n * n].reshape(n, n).copy()))
            eo += n
            uo += n * n
        return out

    def dgemm_tc(self, A, B, transA=False, transB=False, alpha=1.0):
        """FP64-accurate op(A) op(B) on the tensor cores."""
        A = np.ascontiguousarray(A, float)
        B = np.ascontiguousarray(B, float)
        M = A.shape[1] if transA else A.shape[0]
        K = A.shape[0] if transA else A.shape[1]
        N = B.shape[0] if transB else B.shape[1]
        C = np.zeros((M, N))
        _call(lib().nrg_dgemm_tc, self.h, int(transA), int(transB), M, N, K, C_double(alpha),
              _dp(A), A.shape[1], _dp(B), B.shape[1], C_double(0.0), _dp(C), N)
        return C

    def broaden(self, energies, weights, omegas, b):
        e = np.ascontiguousarray(energies, float)
        w = np.ascontiguousarray(weights, float)
        o = np.ascontiguousarray(omegas, float)
        out = np.zeros(len(o))
        _call(lib().nrg_broaden, self.h, _dp(e), _dp(w), C.c_uint64(len(e)), _dp(o),
              C.c_uint64(len(o)), C.c_double(b), _dp(out))
        return out


def broaden_noalloc(energies_ptr, weights_ptr, nbins, omegas_ptr, nomega, b, out_ptr, stream=0):
    """nrg_broaden_noalloc: broadening on caller-owned device buffers (raw
    device addresses of float64 arrays), enqueued on `stream` (a cudaStream_t
    value, 0 = legacy default stream); allocates nothing.  Returns at once:
    synchronize the stream before reading `out`."""
    _call(lib().nrg_broaden_noalloc, C.c_void_p(energies_ptr), C.c_void_p(weights_ptr), C.c_uint64(nbins),
          C.c_void_p(omegas_ptr), C.c_uint64(nomega), C.c_double(b), C.c_void_p(out_ptr),
          C.c_void_p(stream))


class NrgCore:
    """nrgcore<Imp,Bath> on the GPU (nrgcore/nrgcore.hpp)."""

    def __init__(self, engine, impurity, bath, nkeep=1024):
        self.engine = engine
        self._imp = _SiteBuffers(impurity, False)
        self._bath = _SiteBuffers(bath, True)
        self.nops = len(impurity.fdag)
        self.h = C.c_void_p()
        _call(lib().nrg_run_create, engine.h, C.byref(self._imp.desc), C.byref(self._bath.desc),
              C.c_uint64(nkeep), C.byref(self.h))
        engine._adopt(self)

    def close(self):
        if self.h:
            lib().nrg_run_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- the iteration (nrgcore.hpp:65-109, 336-342)
    def set_parameters(self, n=1024):
        _call(lib().nrg_run_set_parameters, self.h, C.c_uint64(n))

    def set_bath(self, bath):
        self._bath_next = _SiteBuffers(bath, True)
        _call(lib().nrg_run_set_bath, self.h, C.byref(self._bath_next.desc))

    def add_bath_site(self, t, rescale):
        t = np.ascontiguousarray(t, float)
        _call(lib().nrg_run_add_site, self.h, _dp(t), len(t), C.c_double(rescale))

    def update_internal_state(self):
        _call(lib().nrg_run_update_state, self.h)

    def checkHigherEnergyDiscarded(self):
        v = C.c_int()
        _call(lib().nrg_run_check_discarded, self.h, C.byref(v))
        return bool(v.value)

    # -- public state (nrgcore.hpp:518-550)
    def info(self):
        i = RunInfo()
        _call(lib().nrg_run_get_info, self.h, C.byref(i))
        return i

    @property
    def nrg_iterations_cnt(self):
        return self.info().iteration

    @property
    def nrg_iterations_min(self):
        return self.info().iteration_min

    @property
    def all_eigenvalue(self):
        n = self.info().n_all
        out = np.zeros(n)
        _call(lib().nrg_run_get_all_eigenvalues, self.h, _dp(out), C.c_uint64(n))
        return out

    @property
    def relativeGroundStateEnergy(self):
        n = self.info().n_relgs
        out = np.zeros(max(n, 1))
        _call(lib().nrg_run_get_relgs, self.h, _dp(out), C.c_uint64(n))
        return out[:n]

    def _sectors(self, which):
        inf = self.info()
        n = inf.n_cur_sectors if which == 0 else inf.n_pre_sectors
        out = np.zeros((max(n, 1), inf.nq), dtype=np.int32)
        _call(lib().nrg_run_get_sectors, self.h, which, _ip(out), C.c_uint64(n))
        return [tuple(int(x) for x in r) for r in out[:n]]

    @property
    def current_sysmQ(self):
        return self._sectors(0)

    @property
    def pre_sysmQ(self):
        return self._sectors(1)

    @property
    def eigenvaluesQ(self):
        inf = self.info()
        nsec = inf.n_cur_sectors if inf.n_cur_sectors else inf.n_pre_sectors
        dims = np.zeros(max(nsec, 1), dtype=np.uint64)
        _call(lib().nrg_run_get_eigenvalues_q, self.h, dims.ctypes.data_as(C.POINTER(C.c_uint64)),
              None, C.c_uint64(0))
        tot = int(dims[:nsec].sum())
        vals = np.zeros(max(tot, 1))
        _call(lib().nrg_run_get_eigenvalues_q, self.h, dims.ctypes.data_as(C.POINTER(C.c_uint64)),
              _dp(vals), C.c_uint64(tot))
        out, o = [], 0
        for d in dims[:nsec]:
            out.append(vals[o:o + int(d)].copy())
            o += int(d)
        return out

    @property
    def kept_counts(self):
        """Sizes of eigenvaluesQ_kept_indices (each is the prefix 0..k-1)."""
        n = self.info().n_pre_sectors
        out = np.zeros(max(n, 1), dtype=np.uint64)
        _call(lib().nrg_run_get_kept, self.h, out.ctypes.data_as(C.POINTER(C.c_uint64)), C.c_uint64(n))
        return [int(x) for x in out[:n]]

    @property
    def eigenvaluesQ_kept_indices(self):
        return [list(range(k)) for k in self.kept_counts]

    @property
    def coupled_nQ_index(self):
        n = self.info().n_cur_sectors or len(self.current_sysmQ)
        counts = np.zeros(max(n, 1), dtype=np.uint64)
        _call(lib().nrg_run_get_coupled, self.h, counts.ctypes.data_as(C.POINTER(C.c_uint64)), None,
              C.c_uint64(0))
        tot = int(counts[:n].sum())
        ent = np.zeros(max(tot, 1), dtype=np.uint64)
        _call(lib().nrg_run_get_coupled, self.h, counts.ctypes.data_as(C.POINTER(C.c_uint64)),
              ent.ctypes.data_as(C.POINTER(C.c_uint64)), C.c_uint64(tot))
        out, o = [], 0
        for c in counts[:n]:
            out.append([int(x) for x in ent[o:o + int(c)]])
            o += int(c)
        return out

    def current_hamiltonQ(self, sector):
        """Eigenvectors (columns) of one sector, row-major n x n."""
        dims = [len(e) for e in self.eigenvaluesQ]
        n = dims[sector]
        out = np.zeros((n, n))
        if n:
            _call(lib().nrg_run_get_eigenvectors, self.h, C.c_int64(sector), _dp(out), C.c_uint64(n * n))
        return out

    def fdag_block(self, ip, i, j):
        """Kept x kept block (i, j) of the rotated f-dagger (get_f_dag_operator)."""
        r, c = C.c_int64(), C.c_int64()
        _call(lib().nrg_run_get_fdag_block, self.h, ip, C.c_int64(i), C.c_int64(j), None,
              C.c_uint64(0), C.byref(r), C.byref(c))
        if r.value == 0 or c.value == 0:
            return None
        out = np.zeros((r.value, c.value))
        _call(lib().nrg_run_get_fdag_block, self.h, ip, C.c_int64(i), C.c_int64(j), _dp(out),
              C.c_uint64(out.size), C.byref(r), C.byref(c))
        return out


def _op_buffers(ops):
    """nrg_op_desc for a list of {(row sector, col sector): block} operators;
    returns (arrays to keep alive, desc)."""
    opi, rows, cols, nr, nc, data = [], [], [], [], [], []
    for ip, d in enumerate(ops):
        for (i, j), m in sorted(d.items()):
            m = np.ascontiguousarray(m, float)
            opi.append(ip)
            rows.append(i)
            cols.append(j)
            nr.append(m.shape[0])
            nc.append(m.shape[1])
            data.append(m.ravel())
    arrs = [np.array(x, dtype=np.int32) for x in (opi, rows, cols, nr, nc)]
    keep = arrs + [np.ascontiguousarray(np.concatenate(data) if data else np.zeros(1))]
    return keep, _OpDesc(len(ops), len(opi), *[_ip(a) for a in arrs], _dp(keep[-1]))


class OperatorSet:
    """Block-sparse operators tracked through the iteration (a device-resident
    vector<qOperator>), given in the run's current previous basis."""

    def __init__(self, run, ops):
        self.run = run
        self.nops = len(ops)
        self._keep, desc = _op_buffers(ops)
        self.h = C.c_void_p()
        _call(lib().nrg_opset_create, run.h, C.byref(desc), C.byref(self.h))
        run.engine._adopt(self)

    def block(self, ip, i, j):
        r, c = C.c_int64(), C.c_int64()
        _call(lib().nrg_opset_get_block, self.h, ip, C.c_int64(i), C.c_int64(j), None, C.c_uint64(0),
              C.byref(r), C.byref(c))
        if r.value == 0 or c.value == 0:
            return None
        out = np.zeros((r.value, c.value))
        _call(lib().nrg_opset_get_block, self.h, ip, C.c_int64(i), C.c_int64(j), _dp(out),
              C.c_uint64(out.size), C.byref(r), C.byref(c))
        return out

    def close(self):
        if self.h:
            lib().nrg_opset_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def update_system_operator(run, opset):
    """update_system_operator(nrg, ops) (sysOperator.hpp:36-133)."""
    _call(lib().nrg_opset_update, opset.h)


class NrgData:
    """Device-resident stand-in for NrgData (nrgData.hpp): saveCurrentData /
    saveqOperator keep the site on the device; loadCurrentData selects it."""

    def __init__(self, run):
        self.run = run

    def saveCurrentData(self, opset=None):
        _call(lib().nrg_run_snapshot, self.run.h, opset.h if opset is not None else None)

    def loadCurrentData(self, iteration=None):
        it = self.run.nrg_iterations_cnt if iteration is None else iteration
        _call(lib().nrg_run_load_snapshot, self.run.h, C.c_int64(it))

    def export(self, path, with_vectors=True):
        """Write every snapshot to `path` in NrgData's group layout
        (nrg_run_export_snapshots; read it back with archive.read / shell)."""
        _call(lib().nrg_run_export_snapshots, self.run.h, os.fsencode(path), int(with_vectors))


class FdmSpectrum:
    """fdmSpectrum<N> (dynamics/fdmSpectrum.hpp): T = 0 as the reference, or
    at a finite temperature after setTemperature(T, thermodynamics)."""

    def __init__(self, run, nops):
        self.run = run
        self.nops = nops
        self.h = C.c_void_p()
        _call(lib().nrg_fdm_create, run.h, nops, C.byref(self.h))
        run.engine._adopt(self)

    def setTemperature(self, T, thermodynamics):
        """Finite-temperature density matrix: each shell's discarded states
        get the Boltzmann weights at T that `thermodynamics` (an
        FdmThermodynamics that has already seen every shell of this backward
        pass) averages with (nrg_fdm_set_temperature)."""
        _call(lib().nrg_fdm_set_temperature, self.h, C.c_double(T), thermodynamics.h)

    def calcSpectrum(self, energy_scale):
        _call(lib().nrg_fdm_calc, self.h, C.c_double(energy_scale))

    def staticExpectation(self):
        """rhoDotStaticOperators summed over the shells so far, per operator
        (<O> at the temperature of the density matrix)."""
        out = np.zeros(self.nops)
        _call(lib().nrg_fdm_get_static, self.h, _dp(out), self.nops)
        return out

    def saveFinalData(self):
        e = np.zeros(FDM_POINTS)
        p = np.zeros((self.nops, FDM_POINTS))
        n = np.zeros((self.nops, FDM_POINTS))
        _call(lib().nrg_fdm_get, self.h, _dp(e), _dp(p), _dp(n), C.c_uint64(FDM_POINTS))
        return {"GreenFnEnergyPoints": e, "GreenFnPositiveWeight": p, "GreenFnNegativeWeight": n}

    def close(self):
        if self.h:
            lib().nrg_fdm_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class FdmThermodynamics:
    """fdmThermodynamics<N> (static/fdmThermodynamics.hpp)."""

    def __init__(self, run, temps):
        self.run = run
        self.temps = np.ascontiguousarray(temps, float)
        self.h = C.c_void_p()
        _call(lib().nrg_thermo_create, run.h, _dp(self.temps), len(self.temps), C.byref(self.h))
        run.engine._adopt(self)
        self.sysops = []

    def setSystemOperator(self, op_index):
        """setSystemOperator (:37-39): operators op_index of the operator set
        saved with each snapshot are averaged as <O>(T)."""
        idx = np.ascontiguousarray(op_index, np.int32)
        _call(lib().nrg_thermo_set_operator, self.h, _ip(idx), len(idx))
        self.sysops = [int(i) for i in idx]

    def calcThermodynamics(self, energy_scale):
        _call(lib().nrg_thermo_calc, self.h, C.c_double(energy_scale))

    def saveFinalData(self):
        s = np.zeros(len(self.temps))
        c = np.zeros(len(self.temps))
        _call(lib().nrg_thermo_final, self.h, _dp(s), _dp(c))
        out = {"temperatureArray": self.temps.copy(), "entropy": s, "specificHeat": c}
        if self.sysops:
            q = np.zeros((len(self.sysops), len(self.temps)))
            _call(lib().nrg_thermo_get_operator, self.h, _dp(q), len(self.sysops), len(self.temps))
            out["qsysOPeratorExpValue"] = q
        return out

    def close(self):
        if self.h:
            lib().nrg_thermo_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def batch_add_site(runs, t, rescale):
    """One add_bath_site for many independent runs with one launch per phase."""
    arr = (C.c_void_p * len(runs))(*[r.h.value for r in runs])
    t = np.ascontiguousarray(t, float).reshape(len(runs), -1)
    rs = np.ascontiguousarray(rescale, float)
    _call(lib().nrg_batch_add_site, arr, len(runs), _dp(t), t.shape[1], _dp(rs))


def update_system_operator_batch(runs, opsets):
    """update_system_operator for several runs' operator sets in shared launches."""
    arr = (C.c_void_p * len(opsets))(*[o.h.value for o in opsets])
    _call(lib().nrg_opset_update_batch, arr, len(opsets))


def fdm_calc_batch(fdms, scales):
    """calcSpectrum for FDM objects of different runs in shared launches."""
    arr = (C.c_void_p * len(fdms))(*[f.h.value for f in fdms])
    sc = np.ascontiguousarray(scales, float)
    _call(lib().nrg_fdm_calc_batch, arr, len(fdms), _dp(sc))


def batch_update_state(runs):
    arr = (C.c_void_p * len(runs))(*[r.h.value for r in runs])
    _call(lib().nrg_batch_update_state, arr, len(runs))


# ---------------------------------------------------------------- serving loop
class _ServerOpts(C.Structure):
    _fields_ = [("max_active", C.c_int), ("hbm_budget_bytes", C.c_uint64), ("workers", C.c_int)]


class _Request(C.Structure):
    _fields_ = [("impurity", C.POINTER(_SiteDesc)), ("bath", C.POINTER(_SiteDesc)), ("nkeep", C.c_uint64),
                ("nsites", C.c_int), ("nt", C.c_int), ("t", C.POINTER(C.c_double)),
                ("rescale", C.POINTER(C.c_double)), ("ops", C.POINTER(_OpDesc)), ("fdm", C.c_int),
                ("ntemps", C.c_int), ("temps", C.POINTER(C.c_double)),
                ("shell_scale", C.POINTER(C.c_double)), ("first_shell_site", C.c_int),
                ("keep_eigenvalues", C.c_int)]


class _ResultInfo(C.Structure):
    _fields_ = [("done", C.c_int), ("status", C.c_int), ("latency_s", C.c_double), ("queue_s", C.c_double),
                ("nsites", C.c_int), ("nops", C.c_int), ("npts", C.c_int), ("ntemps", C.c_int),
                ("n_eig_total", C.c_int64), ("peak_device_bytes", C.c_uint64), ("message", C.c_char * 256)]


class _ServerStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in ("submitted", "completed", "failed", "queued", "max_active_seen",
                                           "ticks")] + \
               [(n, C.c_double) for n in ("busy_s", "p50_latency_s", "p99_latency_s", "mean_latency_s",
                                          "max_latency_s", "footprint_coef")]


class Server:
    """Continuous-batching serving loop (nrg_server_*): whole NRG runs are
    submitted from any thread, admitted by count and HBM budget, stepped
    together one Wilson site per tick, and their backward passes run when
    they finish.  `workers` worker threads each drive one engine (the given
    one and workers - 1 the server creates with its options), so the host
    work of one tick overlaps the GPU work of another.  The given engine must
    not be used elsewhere while it serves."""

    def __init__(self, engine, max_active=16, hbm_budget_bytes=0, workers=1):
        self.engine = engine
        self.h = C.c_void_p()
        opts = _ServerOpts(max_active, hbm_budget_bytes, workers)
        _call(lib().nrg_server_create, engine.h, C.byref(opts), C.byref(self.h))

    def submit(self, impurity, bath, nkeep, t, rescale, ops=None, fdm=False, temps=None, shell_scale=None,
               first_shell_site=0, keep_eigenvalues=False):
        imp = _SiteBuffers(impurity, False)
        bt = _SiteBuffers(bath, True)
        t = np.ascontiguousarray(t, float)
        nsites, nt = t.shape
        rs = np.ascontiguousarray(rescale, float)
        keep = [imp, bt, t, rs]
        opd = None
        if ops is not None:
            k, opd = _op_buffers(ops)
            keep += k
        tp = np.ascontiguousarray(temps if temps is not None else np.zeros(0), float)
        sc = np.ascontiguousarray(shell_scale, float) if shell_scale is not None else None
        keep += [tp, sc]
        req = _Request(C.pointer(imp.desc), C.pointer(bt.desc), nkeep, nsites, nt, _dp(t), _dp(rs),
                       C.pointer(opd) if opd is not None else None, int(fdm), len(tp),
                       _dp(tp) if len(tp) else None, _dp(sc) if sc is not None else None,
                       first_shell_site, int(keep_eigenvalues))
        rid = C.c_uint64()
        _call(lib().nrg_server_submit, self.h, C.byref(req), C.byref(rid))
        return rid.value

    def wait(self, rid, timeout=600.0):
        done = C.c_int()
        _call(lib().nrg_server_wait, self.h, C.c_uint64(rid), C.c_double(timeout), C.byref(done))
        return bool(done.value)

    def info(self, rid):
        inf = _ResultInfo()
        _call(lib().nrg_server_result_info, self.h, C.c_uint64(rid), C.byref(inf))
        return inf

    def result(self, rid, release=True):
        """Results of a finished request; raises NrgError if it failed."""
        inf = self.info(rid)
        if not inf.done:
            raise NrgError(2, "request not finished")
        if inf.status != 0:
            msg = inf.message.decode()
            if release:
                _call(lib().nrg_server_release, self.h, C.c_uint64(rid))
            raise NrgError(inf.status, msg)
        eigs = np.zeros(max(1, inf.n_eig_total))
        counts = np.zeros(max(1, inf.nsites), dtype=np.uint64)
        ep = np.zeros(max(1, inf.npts))
        pos = np.zeros((max(1, inf.nops), max(1, inf.npts)))
        neg = np.zeros_like(pos)
        ent = np.zeros(max(1, inf.ntemps))
        cv = np.zeros_like(ent)
        _call(lib().nrg_server_get_result, self.h, C.c_uint64(rid), _dp(eigs),
              counts.ctypes.data_as(C.POINTER(C.c_uint64)), _dp(ep), _dp(pos), _dp(neg), _dp(ent), _dp(cv))
        out = {"latency_s": inf.latency_s, "queue_s": inf.queue_s, "peak_device_bytes": inf.peak_device_bytes}
        if inf.n_eig_total:
            o, eig = 0, []
            for c in counts[:inf.nsites]:
                eig.append(eigs[o:o + int(c)].copy())
                o += int(c)
            out["eig"] = eig
        if inf.npts:
            out.update({"GreenFnEnergyPoints": ep, "GreenFnPositiveWeight": pos[:inf.nops],
                        "GreenFnNegativeWeight": neg[:inf.nops]})
        if inf.ntemps:
            out.update({"entropy": ent[:inf.ntemps], "specificHeat": cv[:inf.ntemps]})
        if release:
            _call(lib().nrg_server_release, self.h, C.c_uint64(rid))
        return out

    def stats(self, reset=False):
        st = _ServerStats()
        _call(lib().nrg_server_stats, self.h, C.byref(st), int(reset))
        return {n: getattr(st, n) for n, _ in _ServerStats._fields_}

    def close(self):
        if self.h:
            lib().nrg_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
