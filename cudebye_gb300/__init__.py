"""GB300 Debye scattering engine — Python side of the C ABI.

A thin ctypes binding of ``libcudebye.so`` (include/cudebye.h). The names
mirror the reference's host functions in cuDebye-v15.cu so that a caller of
the reference finds each step:

=====================  =========================================  ==========
this module            reference                                  file:line
=====================  =========================================  ==========
``read_deb``           .deb parsing in main()                     :629-833
``channels``           channels = int(rmax/rstep)+2               :732
``k_grid``             2theta and K grid                          :690-698
``Engine.upload``      cudaMalloc/cudaMemcpy of x, y, z           :865-914
``Engine.split_calc_dist``  splitCalcDist + dist/dist2/care_dist2  :88-272
``Engine.histogram``   the pair loop over splitCalcDist           :941-967
``reduce_check``       reduceCheck self-checks                    :360-410
``Engine.atomic_prop`` atomicProp / atomicScatter                 :447-479
``Engine.intensity``   intensity / debyeRowSum, summed over pairs :493-577
``Engine.run_deb``     main(): .deb in, .debx / .debI out          :599-1004
=====================  =========================================  ==========

There is no CPU fallback: importing works without a GPU, but every compute
call needs the compiled library and a CUDA device and raises otherwise.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
# CUDEBYE_LIB names another build of the library (e.g. an installed copy).
LIB_PATH = os.environ.get("CUDEBYE_LIB") or os.path.join(_HERE, "_build",
                                                         "libcudebye.so")
CLI_PATH = os.path.join(_HERE, "_build", "cudebye")

DBX_OK = 0
ERRORS = {
    -1: "DBX_ERR_ARG", -2: "DBX_ERR_CUDA", -3: "DBX_ERR_NOMEM",
    -4: "DBX_ERR_FILE", -5: "DBX_ERR_PARSE", -6: "DBX_ERR_COUNT",
    -7: "DBX_ERR_RANGE", -8: "DBX_ERR_MODEL", -9: "DBX_ERR_TIMEOUT",
    -10: "DBX_ERR_IO", -11: "DBX_ERR_LIMIT",
}
MODES = {"tc": 0, "fp64": 1, "fp32": 2, "plain": 3, "tc3": 4, "tf32": 5}

# Every symbol include/cudebye.h declares (checked by the CPU tests).
EXPORTS = (
    "dbx_create", "dbx_destroy", "dbx_strerror", "dbx_last_error",
    "dbx_device_bytes", "dbx_model_upload", "dbx_model_upload_xyz",
    "dbx_model_free",
    "dbx_pair_histogram", "dbx_pair_histogram_plain", "dbx_histogram",
    "dbx_channels", "dbx_reduce_check",
    "dbx_k_grid", "dbx_atomic_prop", "dbx_intensity", "dbx_pattern",
    "dbx_set_stream", "dbx_set_timing", "dbx_get_timing", "dbx_get_traffic",
    "dbx_run_deb", "dbx_pair_histogram_noalloc", "dbx_patterns",
    "dbx_pattern_errors", "dbx_batch_tuning",
    "dbx_set_graphs", "dbx_server_create", "dbx_server_submit",
    "dbx_server_wait", "dbx_server_stats", "dbx_server_destroy",
    "dbx_check_sqrt", "dbx_xyz2deb", "dbx_xyz2deb_defaults", "dbx_deb_pack",
    "dbx_run_dir", "dbx_curve_index",
)
TIMERS = ("hist", "hist_reduce", "prefactor", "debye", "pass")


class DebyeError(RuntimeError):
    """A DBX_ERR_* status from the engine."""

    def __init__(self, code, msg):
        self.code = code
        super().__init__("%s (%d): %s" % (ERRORS.get(code, "?"), code, msg))


class Species(ctypes.Structure):
    """dbx_species: occupancy, Beq and the 11 scattering-factor parameters."""
    _fields_ = [("occ", ctypes.c_double), ("beq", ctypes.c_double),
                ("a", ctypes.c_double * 5), ("b", ctypes.c_double * 5),
                ("c", ctypes.c_double)]

    @classmethod
    def make(cls, occ, beq, a, b, c):
        s = cls()
        s.occ, s.beq, s.c = float(occ), float(beq), float(c)
        for i in range(5):
            s.a[i] = float(a[i])
            s.b[i] = float(b[i])
        return s


class Request(ctypes.Structure):
    """dbx_request: one pattern request of the server."""
    _fields_ = [("model", ctypes.c_int64),
                ("x", ctypes.POINTER(ctypes.c_float)),
                ("y", ctypes.POINTER(ctypes.c_float)),
                ("z", ctypes.POINTER(ctypes.c_float)),
                ("species_counts", ctypes.POINTER(ctypes.c_int64)),
                ("nspecies", ctypes.c_int),
                ("sp", ctypes.POINTER(Species)),
                ("rstep", ctypes.c_double),
                ("nbins", ctypes.c_int64),
                ("K", ctypes.POINTER(ctypes.c_double)),
                ("nq", ctypes.c_int)]


_lib = None


class XyzDebParams(ctypes.Structure):
    """dbx_xyz2deb_params: the header values of a converted .deb."""
    _fields_ = [("device", ctypes.c_int), ("block", ctypes.c_int),
                ("grid", ctypes.c_int), ("lam", ctypes.c_double),
                ("tt_min", ctypes.c_double), ("tt_max", ctypes.c_double),
                ("tt_step", ctypes.c_double), ("rstep", ctypes.c_double),
                ("intensity", ctypes.c_int), ("distances", ctypes.c_int)]


def load_library(path=None):
    """Load libcudebye.so (built by cudebye_gb300.build); raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            "libcudebye.so not built (%s); run "
            "`python -c 'import __graft_entry__ as g; g.build()'`" % p)
    lib = ctypes.CDLL(p)
    c_p = ctypes.c_void_p
    i64p = ctypes.POINTER(ctypes.c_int64)
    dp = ctypes.POINTER(ctypes.c_double)
    fp = ctypes.POINTER(ctypes.c_float)
    sig = {
        "dbx_create": (ctypes.c_int, [ctypes.POINTER(c_p), ctypes.c_int,
                                      ctypes.c_size_t]),
        "dbx_destroy": (ctypes.c_int, [c_p]),
        "dbx_strerror": (ctypes.c_char_p, [ctypes.c_int]),
        "dbx_last_error": (ctypes.c_char_p, [c_p]),
        "dbx_device_bytes": (ctypes.c_size_t, [c_p]),
        "dbx_model_upload": (ctypes.c_int, [c_p, fp, fp, fp, i64p,
                                            ctypes.c_int, i64p]),
        "dbx_model_upload_xyz": (ctypes.c_int, [c_p, fp, i64p, ctypes.c_int,
                                                i64p]),
        "dbx_model_free": (ctypes.c_int, [c_p, ctypes.c_int64]),
        "dbx_pair_histogram": (ctypes.c_int, [c_p, ctypes.c_int64, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_double,
                                              ctypes.c_int64, i64p]),
        "dbx_pair_histogram_plain": (ctypes.c_int, [
            c_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_double,
            ctypes.c_int64, i64p]),
        "dbx_histogram": (ctypes.c_int, [c_p, ctypes.c_int64, ctypes.c_double,
                                         ctypes.c_int64, i64p]),
        "dbx_channels": (ctypes.c_int64, [ctypes.c_double, ctypes.c_double]),
        "dbx_curve_index": (ctypes.c_int64, [ctypes.c_uint32] * 3 + [ctypes.c_int]),
        "dbx_reduce_check": (ctypes.c_int, [i64p, ctypes.c_int64,
                                            ctypes.c_double, ctypes.c_int64,
                                            ctypes.c_int64, ctypes.c_int, i64p]),
        "dbx_k_grid": (ctypes.c_int, [ctypes.c_double] * 4 + [dp, dp]),
        "dbx_atomic_prop": (ctypes.c_int, [c_p, ctypes.POINTER(Species),
                                           ctypes.POINTER(Species), dp,
                                           ctypes.c_int, dp]),
        "dbx_intensity": (ctypes.c_int, [c_p, ctypes.c_int64, ctypes.c_double,
                                         ctypes.c_int64,
                                         ctypes.POINTER(Species), dp,
                                         ctypes.c_int, ctypes.c_int, dp]),
        "dbx_pattern": (ctypes.c_int, [c_p, ctypes.c_int64, ctypes.c_double,
                                       ctypes.c_int64,
                                       ctypes.POINTER(Species), dp,
                                       ctypes.c_int, ctypes.c_int, dp]),
        "dbx_set_stream": (ctypes.c_int, [c_p, c_p]),
        "dbx_set_timing": (ctypes.c_int, [c_p, ctypes.c_int]),
        "dbx_get_timing": (ctypes.c_int, [c_p, dp]),
        "dbx_get_traffic": (ctypes.c_int, [c_p, i64p]),
        "dbx_run_deb": (ctypes.c_int, [c_p, ctypes.c_char_p, ctypes.c_char_p,
                                       ctypes.c_int]),
        "dbx_run_dir": (ctypes.c_int, [c_p, ctypes.c_char_p, ctypes.c_char_p,
                                       ctypes.c_int]),
        "dbx_patterns": (ctypes.c_int, [c_p, i64p, ctypes.c_int,
                                        ctypes.c_double, i64p,
                                        ctypes.POINTER(Species), dp,
                                        ctypes.c_int, ctypes.c_int, dp]),
        "dbx_pattern_errors": (ctypes.c_int, [c_p, i64p, ctypes.c_int,
                                              ctypes.c_double, i64p,
                                              ctypes.POINTER(Species), dp,
                                              ctypes.c_int, dp, ctypes.c_int,
                                              dp]),
        "dbx_set_graphs": (ctypes.c_int, [c_p, ctypes.c_int]),
        "dbx_batch_tuning": (ctypes.c_int, [c_p, dp]),
        "dbx_check_sqrt": (ctypes.c_int, [c_p, ctypes.c_uint32, ctypes.c_uint32,
                                          i64p]),
        "dbx_server_create": (ctypes.c_int, [ctypes.POINTER(c_p), ctypes.c_int,
                                             ctypes.c_size_t]),
        "dbx_server_submit": (ctypes.c_int, [c_p, ctypes.POINTER(Request),
                                             i64p]),
        "dbx_server_wait": (ctypes.c_int, [c_p, ctypes.c_int64, dp,
                                           ctypes.c_int, i64p, dp]),
        "dbx_server_stats": (ctypes.c_int, [c_p, i64p]),
        "dbx_server_destroy": (ctypes.c_int, [c_p]),
        "dbx_pair_histogram_noalloc": (ctypes.c_int, [
            c_p, c_p, c_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
            ctypes.c_int64, ctypes.c_double, ctypes.c_int64, c_p, c_p]),
        "dbx_xyz2deb_defaults": (None, [ctypes.POINTER(XyzDebParams)]),
        "dbx_deb_pack": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p,
                                        ctypes.c_char_p, ctypes.c_size_t]),
        "dbx_xyz2deb": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p,
                                       ctypes.POINTER(XyzDebParams),
                                       ctypes.c_char_p, ctypes.c_char_p,
                                       ctypes.c_size_t]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _ptr(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


# ---- host-only helpers (no GPU needed) ------------------------------------

def channels(rmax, rstep):
    """int(rmax/rstep)+2 (cuDebye-v15.cu:732)."""
    return int(rmax / rstep) + 2


def curve_index(x, y, z, bits):
    """Position of grid cell (x, y, z) along the Hilbert curve that orders
    each species' atoms into tiles (dbx_curve_index; -1 if out of range)."""
    return int(load_library().dbx_curve_index(x, y, z, bits))


def k_grid(lam, tt_min, tt_max, tt_step):
    """(2theta, K) with K = 4 pi sin(2theta/2 pi/180)/lambda
    (cuDebye-v15.cu:690-698)."""
    n = int((tt_max - tt_min) / tt_step) + 1
    tt = tt_min + np.arange(n, dtype=np.float64) * tt_step
    K = 4 * np.pi * np.sin(tt / 2 * np.pi / 180) / lam
    return tt, K


def pair_list(nspecies):
    """Species pairs in the reference's loop order (cuDebye-v15.cu:941-942)."""
    return [(r, c) for r in range(nspecies) for c in range(r, nspecies)]


def reduce_check(counts, rstep, n_row, n_col, diag):
    """Self-checks of reduceCheck (cuDebye-v15.cu:360-410) on one histogram.

    Returns dict(expected, observed, bin0, collisions)."""
    counts = np.asarray(counts, dtype=np.int64)
    r = np.arange(counts.size) * rstep
    expected = (n_col * n_row - n_row) // 2 + n_col if diag else n_col * n_row
    below = int(counts[r < 0.25].sum())
    return dict(expected=int(expected), observed=int(counts.sum()),
                bin0=int(counts[0]),
                collisions=max(0, below - n_col) if diag else below)


class DebFile:
    """Contents of a .deb file (cuDebye-v15.cu:629-833)."""

    def __init__(self):
        self.device = self.block = self.grid = 0
        self.lam = self.tt_min = self.tt_max = self.tt_step = 0.0
        self.rmax = self.rstep = 0.0
        self.hist = 0
        self.names, self.counts, self.species = [], [], []
        self.xyz = np.zeros((0, 3), np.float32)


def xyz2deb(xyz_path, table_path, deb_path=None, **params):
    """The reference's Matlab converter (Matlab/xyz2deb.m): write a .deb from
    an "element x y z [occ [Beq]]" file and a Waasmaier-Kirfel table in the
    RIETAN layout. Keyword arguments override the script's defaults (device,
    block, grid, lam, tt_min, tt_max, tt_step, rstep, intensity,
    distances). Returns the .deb path. Needs no GPU."""
    lib = load_library()
    p = XyzDebParams()
    lib.dbx_xyz2deb_defaults(ctypes.byref(p))
    for k, v in params.items():
        if not hasattr(p, k):
            raise TypeError("unknown xyz2deb parameter %r" % k)
        setattr(p, k, v)
    msg = ctypes.create_string_buffer(512)
    rc = lib.dbx_xyz2deb(xyz_path.encode(), table_path.encode(),
                         ctypes.byref(p),
                         deb_path.encode() if deb_path else None, msg, 512)
    if rc != DBX_OK:
        raise DebyeError(rc, msg.value.decode(errors="replace"))
    return deb_path or (xyz_path[:-3] + "deb")


def deb_pack(deb_path, out_path):
    """Write the binary form of a .deb (dbx_deb_pack). Needs no GPU."""
    lib = load_library()
    msg = ctypes.create_string_buffer(512)
    rc = lib.dbx_deb_pack(deb_path.encode(), out_path.encode(), msg, 512)
    if rc != DBX_OK:
        raise DebyeError(rc, msg.value.decode(errors="replace"))
    return out_path


def read_debb(path):
    """Parse the binary form written by deb_pack into a DebFile."""
    import struct
    with open(path, "rb") as f:
        b = f.read()
    if b[:8] != b"DBXDEB1\0":
        raise DebyeError(-5, "not a binary .deb")
    d = DebFile()
    d.device, d.block, d.grid, d.hist = struct.unpack_from("<4i", b, 8)
    (d.lam, d.tt_min, d.tt_max, d.tt_step, d.rmax,
     d.rstep) = struct.unpack_from("<6d", b, 24)
    nsp, _ = struct.unpack_from("<2i", b, 72)
    pos = 80
    d.counts, d.names, d.species = [], [], []
    for _ in range(nsp):
        n, = struct.unpack_from("<q", b, pos)
        name = b[pos + 8:pos + 40].split(b"\0")[0].decode()
        v = struct.unpack_from("<13d", b, pos + 40)
        pos += 144
        d.counts.append(n)
        d.names.append(name)
        d.species.append(Species.make(v[0], v[1], v[2:7], v[7:12], v[12]))
    N = sum(d.counts)
    xyz = np.frombuffer(b, np.float32, 3 * N, pos).reshape(3, N)
    d.xyz = np.ascontiguousarray(xyz.T)
    return d


def read_deb(path):
    """Parse a .deb file into a DebFile (same rules as the engine's reader:
    header lines 1-4, one species line each, then x y z per non-blank line;
    coordinates rounded to FP32 like istringstream >> float)."""
    if not os.path.exists(path):
        raise DebyeError(-4, ">>%s<< does not exist" % path)
    with open(path, "r") as f:
        lines = f.read().split("\n")
    d = DebFile()
    try:
        h1, h2, h3, h4 = (lines[i].split() for i in range(4))
        d.device, d.block, d.grid = int(h1[0]), int(h1[1]), int(h1[2])
        d.lam, d.tt_min, d.tt_max, d.tt_step = map(float, h2[:4])
        d.rmax, d.rstep, d.hist = float(h3[0]), float(h3[1]), int(h3[2])
        if d.hist not in (1, 2):
            d.hist = 0
        p = int(h4[0])
        for i in range(p):
            t = lines[4 + i].split()
            d.counts.append(int(t[0]))
            d.names.append(t[1])
            v = [float(s) for s in t[2:15]]
            d.species.append(Species.make(v[0], v[1], v[2:7], v[7:12], v[12]))
    except (IndexError, ValueError) as e:
        raise DebyeError(-5, "malformed .deb header: %s" % e)
    rows = [l for l in lines[4 + p:] if l.strip()]
    if len(rows) != sum(d.counts):
        raise DebyeError(-6, "Number of extracted Atoms (%d) doesn't match the "
                         "number specified in the preamble (%d)"
                         % (len(rows), sum(d.counts)))
    try:
        d.xyz = np.array([[float(v) for v in r.split()[:3]] for r in rows],
                         dtype=np.float32).reshape(-1, 3)
    except ValueError as e:
        raise DebyeError(-5, "malformed coordinate line: %s" % e)
    return d


# ---- the engine (GPU) ------------------------------------------------------

class Model:
    """Handle of a model resident on the device."""

    def __init__(self, engine, mid, counts):
        self.engine, self.id, self.counts = engine, mid, list(counts)

    @property
    def nspecies(self):
        return len(self.counts)

    def free(self):
        if self.id is not None:
            self.engine._check(self.engine.lib.dbx_model_free(self.engine.ctx,
                                                              self.id))
            self.id = None


class Engine:
    """A device context (dbx_ctx) on one GPU."""

    def __init__(self, device=0, hbm_budget=0, lib_path=None):
        self.lib = load_library(lib_path)
        self.ctx = ctypes.c_void_p()
        rc = self.lib.dbx_create(ctypes.byref(self.ctx), device, hbm_budget)
        if rc != DBX_OK:
            raise DebyeError(rc, "dbx_create(device=%d) failed" % device)

    def close(self):
        if self.ctx:
            self.lib.dbx_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != DBX_OK:
            msg = self.lib.dbx_last_error(self.ctx) or b""
            raise DebyeError(rc, msg.decode(errors="replace"))

    @property
    def device_bytes(self):
        return int(self.lib.dbx_device_bytes(self.ctx))

    def upload(self, xyz, counts):
        """Upload FP32 coordinates (n x 3, grouped by species in order)."""
        # interleaved [n][3] as given (dbx_model_upload_xyz): no transpose
        xyz = np.ascontiguousarray(np.asarray(xyz, dtype=np.float32).reshape(-1, 3))
        c = np.ascontiguousarray(counts, dtype=np.int64)
        if int(c.sum()) != xyz.shape[0]:
            raise DebyeError(-6, "species counts do not sum to the atom count")
        mid = ctypes.c_int64()
        self._check(self.lib.dbx_model_upload_xyz(
            self.ctx, _ptr(xyz, ctypes.c_float), _ptr(c, ctypes.c_int64), len(c),
            ctypes.byref(mid)))
        return Model(self, mid.value, c)

    def upload_planes(self, x, y, z, counts):
        """Upload SoA coordinate planes (dbx_model_upload, the reference's
        x[], y[], z[] arrays)."""
        x, y, z = (np.ascontiguousarray(v, dtype=np.float32) for v in (x, y, z))
        c = np.ascontiguousarray(counts, dtype=np.int64)
        if not (x.size == y.size == z.size == int(c.sum())):
            raise DebyeError(-6, "species counts do not sum to the atom count")
        mid = ctypes.c_int64()
        self._check(self.lib.dbx_model_upload(
            self.ctx, _ptr(x, ctypes.c_float), _ptr(y, ctypes.c_float),
            _ptr(z, ctypes.c_float), _ptr(c, ctypes.c_int64), len(c),
            ctypes.byref(mid)))
        return Model(self, mid.value, c)

    def split_calc_dist(self, model, row, col, rstep, nbins):
        """int64 histogram of species pair (row, col) (splitCalcDist)."""
        out = np.zeros(nbins, dtype=np.int64)
        self._check(self.lib.dbx_pair_histogram(
            self.ctx, model.id, row, col, rstep, nbins,
            _ptr(out, ctypes.c_int64)))
        return out

    def split_calc_dist_plain(self, model, row, col, rstep, nbins):
        """The same histogram from the plain unbatched FP32 GPU form (one
        thread per pair, global atomics; dbx_pair_histogram_plain)."""
        out = np.zeros(nbins, dtype=np.int64)
        self._check(self.lib.dbx_pair_histogram_plain(
            self.ctx, model.id, row, col, rstep, nbins,
            _ptr(out, ctypes.c_int64)))
        return out

    def histogram(self, model, rstep, nbins):
        """All pair histograms [npairs, nbins] in the reference's pair order."""
        p = model.nspecies
        out = np.zeros((p * (p + 1) // 2, nbins), dtype=np.int64)
        self._check(self.lib.dbx_histogram(self.ctx, model.id, rstep, nbins,
                                           _ptr(out, ctypes.c_int64)))
        return out

    def atomic_prop(self, sp_a, sp_b, K):
        """Per-q prefactor of one pair (atomicProp)."""
        K = np.ascontiguousarray(K, dtype=np.float64)
        out = np.zeros(K.size, dtype=np.float64)
        self._check(self.lib.dbx_atomic_prop(
            self.ctx, ctypes.byref(sp_a), ctypes.byref(sp_b),
            _ptr(K, ctypes.c_double), K.size, _ptr(out, ctypes.c_double)))
        return out

    def intensity(self, model, rstep, nbins, species, K, mode="tc"):
        """I(K) summed over all species pairs (intensity, per pair loop)."""
        K = np.ascontiguousarray(K, dtype=np.float64)
        sp = (Species * len(species))(*species)
        out = np.zeros(K.size, dtype=np.float64)
        self._check(self.lib.dbx_intensity(
            self.ctx, model.id, rstep, nbins, sp, _ptr(K, ctypes.c_double),
            K.size, MODES[mode], _ptr(out, ctypes.c_double)))
        return out

    def pattern(self, model, rstep, nbins, species, K, mode="tc", out=None):
        """One full pattern: histograms recomputed, then the Debye sum."""
        K = np.ascontiguousarray(K, dtype=np.float64)
        sp = (Species * len(species))(*species)
        if out is None:
            out = np.zeros(K.size, dtype=np.float64)
        self._check(self.lib.dbx_pattern(
            self.ctx, model.id, rstep, nbins, sp, _ptr(K, ctypes.c_double),
            K.size, MODES[mode], _ptr(out, ctypes.c_double)))
        return out

    def batch_tuning(self):
        """The batch autotuner's choice for the last patterns() plan
        (dbx_batch_tuning)."""
        out = np.zeros(8)
        self._check(self.lib.dbx_batch_tuning(self.ctx, _ptr(out, ctypes.c_double)))
        return {"tasks": int(out[0]), "tasks_per_sm": float(out[1]),
                "multi_window": bool(out[2]), "rowq": float(out[3]),
                "geometry": ("sampled", "disjoint", "overlap")[int(out[4])],
                "shapes_timed": int(out[5]), "task_counts_timed": int(out[6]),
                "hist_ms": float(out[7])}

    def patterns(self, models, rstep, nbins, species, K, mode="tc", out=None):
        """Full patterns of several resident models in one pass
        (dbx_patterns): nbins per model, species = concatenated per-model
        species lists (model order). Returns I[nmodels, nq]."""
        K = np.ascontiguousarray(K, dtype=np.float64)
        ids = np.ascontiguousarray([m.id for m in models], dtype=np.int64)
        nb = np.ascontiguousarray(nbins, dtype=np.int64)
        sp = (Species * len(species))(*species)
        if out is None:
            out = np.zeros((len(models), K.size), dtype=np.float64)
        self._check(self.lib.dbx_patterns(
            self.ctx, _ptr(ids, ctypes.c_int64), len(models), rstep,
            _ptr(nb, ctypes.c_int64), sp, _ptr(K, ctypes.c_double), K.size,
            MODES[mode], _ptr(out, ctypes.c_double)))
        return out

    def pattern_errors(self, models, rstep, nbins, species, K, I, q_stride=10):
        """Max relative error of each row of I (patterns() of the same
        arguments) against the FP64 direct sum at every q_stride-th q
        (dbx_pattern_errors). Returns an array [nmodels]."""
        K = np.ascontiguousarray(K, dtype=np.float64)
        I = np.ascontiguousarray(I, dtype=np.float64)
        ids = np.ascontiguousarray([m.id for m in models], dtype=np.int64)
        nb = np.ascontiguousarray(nbins, dtype=np.int64)
        sp = (Species * len(species))(*species)
        out = np.zeros(len(models), dtype=np.float64)
        self._check(self.lib.dbx_pattern_errors(
            self.ctx, _ptr(ids, ctypes.c_int64), len(models), rstep,
            _ptr(nb, ctypes.c_int64), sp, _ptr(K, ctypes.c_double), K.size,
            _ptr(I, ctypes.c_double), int(q_stride), _ptr(out, ctypes.c_double)))
        return out

    def check_sqrt(self, lo_bits=0, hi_bits=0x7F800000):
        """Device check of the histogram kernels' square root against the
        IEEE one over the floats with bits in [lo_bits, hi_bits]:
        (checked, mismatches, smallest mismatching bits or -1)."""
        out = np.zeros(3, np.int64)
        self._check(self.lib.dbx_check_sqrt(self.ctx, lo_bits, hi_bits,
                                            _ptr(out, ctypes.c_int64)))
        return int(out[0]), int(out[1]), int(out[2])

    def set_graphs(self, on=True):
        self._check(self.lib.dbx_set_graphs(self.ctx, int(on)))

    def set_stream(self, stream_handle):
        """Launch on a caller's cudaStream_t (int handle, e.g.
        torch.cuda.Stream().cuda_stream); None = the context's own."""
        self._check(self.lib.dbx_set_stream(
            self.ctx, ctypes.c_void_p(stream_handle) if stream_handle else None))

    def set_timing(self, on=True):
        self._check(self.lib.dbx_set_timing(self.ctx, int(on)))

    def timing(self):
        """{phase: ms} of the last call (CUDA events on the launch stream)."""
        out = np.zeros(len(TIMERS))
        self._check(self.lib.dbx_get_timing(self.ctx,
                                            _ptr(out, ctypes.c_double)))
        return dict(zip(TIMERS, out.tolist()))

    def traffic(self):
        """(h2d_bytes, d2h_bytes) copied by this context so far."""
        out = np.zeros(2, np.int64)
        self._check(self.lib.dbx_get_traffic(self.ctx,
                                             _ptr(out, ctypes.c_int64)))
        return int(out[0]), int(out[1])

    def run_deb(self, path, out_prefix=None, verbose=False):
        """The reference's main(): .deb in, .debx/.debI written."""
        self._check(self.lib.dbx_run_deb(
            self.ctx, path.encode(),
            out_prefix.encode() if out_prefix else None, int(verbose)))

    def run_dir(self, folder, table=None, verbose=False):
        """The reference's multisim: convert .xyz without .deb (with a
        scattering-factor table), compute every .deb without .debI."""
        self._check(self.lib.dbx_run_dir(
            self.ctx, folder.encode(), table.encode() if table else None,
            int(verbose)))


class Server:
    """A pattern server (dbx_server): thread-safe submit / wait."""

    def __init__(self, device=0, hbm_budget=0, lib_path=None):
        self.lib = load_library(lib_path)
        self.srv = ctypes.c_void_p()
        rc = self.lib.dbx_server_create(ctypes.byref(self.srv), device,
                                        hbm_budget)
        if rc != DBX_OK:
            raise DebyeError(rc, "dbx_server_create failed")

    def submit(self, species, rstep, nbins, K, xyz=None, counts=None,
               model=0):
        """New model (xyz, counts) or re-score of a resident model id.
        Returns a ticket."""
        K = np.ascontiguousarray(K, dtype=np.float64)
        sp = (Species * len(species))(*species)
        r = Request()
        r.model = int(model)
        keep = [K, sp]
        if not model:
            xyz = np.asarray(xyz, np.float32).reshape(-1, 3)
            cols = [np.ascontiguousarray(xyz[:, i]) for i in range(3)]
            c = np.ascontiguousarray(counts, dtype=np.int64)
            keep += cols + [c]
            r.x, r.y, r.z = (_ptr(a, ctypes.c_float) for a in cols)
            r.species_counts = _ptr(c, ctypes.c_int64)
        r.nspecies = len(species)
        r.sp = sp
        r.rstep = rstep
        r.nbins = int(nbins)
        r.K = _ptr(K, ctypes.c_double)
        r.nq = K.size
        t = ctypes.c_int64()
        rc = self.lib.dbx_server_submit(self.srv, ctypes.byref(r),
                                        ctypes.byref(t))
        if rc != DBX_OK:
            raise DebyeError(rc, "submit rejected")
        return t.value

    def wait(self, ticket, nq):
        """(I, model_id, latency_ms) of a ticket; raises on a failed request."""
        out = np.zeros(nq, dtype=np.float64)
        mid = ctypes.c_int64()
        lat = ctypes.c_double()
        rc = self.lib.dbx_server_wait(self.srv, ticket,
                                      _ptr(out, ctypes.c_double), nq,
                                      ctypes.byref(mid), ctypes.byref(lat))
        if rc != DBX_OK:
            raise DebyeError(rc, "request %d failed" % ticket)
        return out, mid.value, lat.value

    def stats(self):
        out = np.zeros(6, np.int64)
        self.lib.dbx_server_stats(self.srv, _ptr(out, ctypes.c_int64))
        return dict(zip(("rounds", "completed", "resident_models",
                         "device_bytes", "evictions", "lane_reserve"),
                        out.tolist()))

    def close(self):
        if self.srv:
            self.lib.dbx_server_destroy(self.srv)
            self.srv = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
