"""ctypes binding of the CPU oracle (oracle.c).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm, as the checker or as the timed CPU
baseline. The engine never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liborc.so")
CLI = os.path.join(BUILD, "orc_debye")
# The reference program (cuDebye-v15.cu built by `make -C oracle ref`)
REF_BIN = os.path.join(HERE, "_ref", "cudebye_ref")

_lib = None


def build():
    """make -C oracle (gcc, -ffp-contract=off)."""
    r = subprocess.run(["make", "-s", "-C", HERE], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def build_ref_start():
    """Start `make -C oracle ref` (nvcc, about 20 s) in the background;
    finish with build_ref_finish(). Nothing is built where neither the
    reference's source nor its edited copy is present."""
    return subprocess.Popen(["make", "-s", "-C", HERE, "ref"],
                            stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                            text=True)


def build_ref_finish(proc):
    """Wait for build_ref_start's make; returns REF_BIN if it exists. A
    failed build leaves the reference program's tests skipped, not the
    engine's build failed, so its output is printed."""
    out, _ = proc.communicate()
    if proc.returncode != 0:
        print("reference program build failed:\n" + out)
    return REF_BIN if os.path.exists(REF_BIN) else None


def lib():
    global _lib
    if _lib is None:
        if not (os.path.exists(LIB) and os.path.exists(CLI)):
            build()
        L = ctypes.CDLL(LIB)
        f32p = ctypes.POINTER(ctypes.c_float)
        i64p = ctypes.POINTER(ctypes.c_int64)
        dp = ctypes.POINTER(ctypes.c_double)
        i64 = ctypes.c_int64
        L.orc_inv_rstep.restype = ctypes.c_float
        L.orc_inv_rstep.argtypes = [ctypes.c_double]
        L.orc_channels.restype = i64
        L.orc_channels.argtypes = [ctypes.c_double, ctypes.c_double]
        L.orc_pair_bin.restype = i64
        L.orc_pair_bin.argtypes = [ctypes.c_float] * 7
        L.orc_block_histogram.restype = i64
        L.orc_block_histogram.argtypes = [f32p, f32p, f32p, i64, i64, i64, i64,
                                          ctypes.c_int, ctypes.c_float, i64p,
                                          i64, ctypes.c_int, i64]
        L.orc_n_two_theta.restype = ctypes.c_int
        L.orc_n_two_theta.argtypes = [ctypes.c_double] * 3
        L.orc_k_grid.restype = None
        L.orc_k_grid.argtypes = [ctypes.c_double] * 3 + [ctypes.c_int, dp, dp]
        L.orc_prefactor.restype = None
        L.orc_prefactor.argtypes = ([dp, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, dp, dp, ctypes.c_double]
                                    + [ctypes.c_double, ctypes.c_double, dp, dp,
                                       ctypes.c_double, dp])
        L.orc_debye_accumulate.restype = None
        L.orc_debye_accumulate.argtypes = [dp, ctypes.c_int, i64p, i64,
                                           ctypes.c_double, dp, dp,
                                           ctypes.c_int, ctypes.c_int]
        L.orc_debye_rowsum.restype = None
        L.orc_debye_rowsum.argtypes = [dp, ctypes.c_int, i64p, i64,
                                       ctypes.c_double, dp, ctypes.c_int]
        L.orc_deb_read.restype = ctypes.c_int
        L.orc_deb_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(OrcDeb)]
        L.orc_deb_free.restype = None
        L.orc_deb_free.argtypes = [ctypes.POINTER(OrcDeb)]
        _lib = L
    return _lib


class OrcSpecies(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("name", ctypes.c_char * 32),
                ("occ", ctypes.c_double), ("beq", ctypes.c_double),
                ("a", ctypes.c_double * 5), ("b", ctypes.c_double * 5),
                ("c", ctypes.c_double)]


class OrcDeb(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("block", ctypes.c_int),
                ("grid", ctypes.c_int), ("lam", ctypes.c_double),
                ("tt_min", ctypes.c_double), ("tt_max", ctypes.c_double),
                ("tt_step", ctypes.c_double), ("rmax", ctypes.c_double),
                ("rstep", ctypes.c_double), ("hist", ctypes.c_int),
                ("nspecies", ctypes.c_int),
                ("sp", ctypes.POINTER(OrcSpecies)), ("natoms", ctypes.c_int64),
                ("x", ctypes.POINTER(ctypes.c_float)),
                ("y", ctypes.POINTER(ctypes.c_float)),
                ("z", ctypes.POINTER(ctypes.c_float))]


def read_deb(path):
    """The oracle's .deb parser (orc_deb_read): (header dict, species list
    of dicts, float32 [N, 3] coordinates); raises on a parse error."""
    d = OrcDeb()
    rc = lib().orc_deb_read(path.encode(), ctypes.byref(d))
    if rc != 0:
        raise RuntimeError("orc_deb_read(%s) = %d" % (path, rc))
    try:
        hdr = {k: getattr(d, k) for k in ("device", "block", "grid", "lam",
                                          "tt_min", "tt_max", "tt_step",
                                          "rmax", "rstep", "hist")}
        sp = [{"n": d.sp[i].n, "name": d.sp[i].name.decode(),
               "occ": d.sp[i].occ, "beq": d.sp[i].beq,
               "a": list(d.sp[i].a), "b": list(d.sp[i].b), "c": d.sp[i].c}
              for i in range(d.nspecies)]
        n = d.natoms
        xyz = np.empty((n, 3), np.float32)
        for c, arr in enumerate((d.x, d.y, d.z)):
            if n:
                xyz[:, c] = np.ctypeslib.as_array(arr, shape=(n,))
        return hdr, sp, xyz
    finally:
        lib().orc_deb_free(ctypes.byref(d))


def _p(a, ct):
    return a.ctypes.data_as(ctypes.POINTER(ct))


def inv_rstep(rstep):
    return lib().orc_inv_rstep(rstep)


def channels(rmax, rstep):
    return lib().orc_channels(rmax, rstep)


def pair_bin(a, b, rstep):
    return lib().orc_pair_bin(*map(float, a), *map(float, b), inv_rstep(rstep))


def block_histogram(xyz, a0, na, b0, nb, diag, rstep, nbins, threads=0,
                    row_stride=1):
    """(hist, out_of_range) of one species block (cuDebye-v15.cu:88-146)."""
    xyz = np.asarray(xyz, np.float32)
    x = np.ascontiguousarray(xyz[:, 0])
    y = np.ascontiguousarray(xyz[:, 1])
    z = np.ascontiguousarray(xyz[:, 2])
    h = np.zeros(nbins, np.int64)
    bad = lib().orc_block_histogram(
        _p(x, ctypes.c_float), _p(y, ctypes.c_float), _p(z, ctypes.c_float),
        a0, na, b0, nb, int(diag), inv_rstep(rstep), _p(h, ctypes.c_int64),
        nbins, threads, row_stride)
    return h, bad


def model_histograms(xyz, counts, rstep, nbins, threads=0):
    """All pair histograms [npairs, nbins] in the reference's pair order."""
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(int)
    out, bad = [], 0
    for r in range(len(counts)):
        for c in range(r, len(counts)):
            h, b = block_histogram(xyz, starts[r], counts[r], starts[c],
                                   counts[c], r == c, rstep, nbins, threads)
            out.append(h)
            bad += b
    return np.array(out).reshape(-1, nbins), bad


def k_grid(lam, tt_min, tt_max, tt_step):
    n = lib().orc_n_two_theta(tt_min, tt_max, tt_step)
    tt = np.zeros(n)
    K = np.zeros(n)
    lib().orc_k_grid(lam, tt_min, tt_step, n, _p(tt, ctypes.c_double),
                     _p(K, ctypes.c_double))
    return tt, K


def prefactor(K, s1, s2):
    """s1, s2: objects with occ, beq, a[5], b[5], c."""
    K = np.ascontiguousarray(K, np.float64)
    ff = np.zeros(K.size)
    a1, b1 = np.array(list(s1.a), float), np.array(list(s1.b), float)
    a2, b2 = np.array(list(s2.a), float), np.array(list(s2.b), float)
    lib().orc_prefactor(_p(K, ctypes.c_double), K.size, s1.occ, s1.beq,
                        _p(a1, ctypes.c_double), _p(b1, ctypes.c_double), s1.c,
                        s2.occ, s2.beq, _p(a2, ctypes.c_double),
                        _p(b2, ctypes.c_double), s2.c, _p(ff, ctypes.c_double))
    return ff


def rowsum(K, hist, rstep, threads=0):
    """S[q] = sum_k m_k sinc(K r_k) over non-zero bins (FP64)."""
    K = np.ascontiguousarray(K, np.float64)
    h = np.ascontiguousarray(hist, np.int64)
    S = np.zeros(K.size)
    lib().orc_debye_rowsum(_p(K, ctypes.c_double), K.size,
                           _p(h, ctypes.c_int64), h.size, rstep,
                           _p(S, ctypes.c_double), threads)
    return S


def intensity(K, hists, species, rstep, threads=0, q_stride=1):
    """I[q] = sum over pairs of ff_pair * rowsum (the reference's pair loop)."""
    K = np.ascontiguousarray(K, np.float64)
    I = np.zeros(K.size)
    P = len(species)
    p = 0
    for r in range(P):
        for c in range(r, P):
            ff = prefactor(K, species[r], species[c])
            h = np.ascontiguousarray(hists[p], np.int64)
            lib().orc_debye_accumulate(_p(K, ctypes.c_double), K.size,
                                       _p(h, ctypes.c_int64), h.size, rstep,
                                       _p(ff, ctypes.c_double),
                                       _p(I, ctypes.c_double), threads,
                                       q_stride)
            p += 1
    return I


def run_deb(deb_path, prefix, threads=0):
    """The whole-file oracle run (orc_debye)."""
    lib()
    r = subprocess.run([CLI, deb_path, prefix, str(threads)],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("orc_debye failed: " + r.stdout + r.stderr)
