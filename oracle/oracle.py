"""ctypes binding for the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this module.  It builds oracle/pp_oracle.cpp (a plain C++/OpenMP
restatement of PARAPROBE's descriptive-statistics path) into
oracle/_build/libppo.so and exposes it with numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libppo.so")
SRC = os.path.join(HERE, "pp_oracle.cpp")

RDF, NN1, RIPK, MKNN, CNTNB = 1, 2, 4, 8, 32

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with the reference's float semantics (no FMA
    contraction) for the host this runs on."""
    import platform
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "machine.txt")
    if not os.path.exists(stamp) or open(stamp).read().strip() != platform.machine():
        force = True
        with open(stamp, "w") as f:
            f.write(platform.machine() + "\n")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp"
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off",
                               "-fPIC", "-shared", "-o", tmp, SRC])
        os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        f32p = np.ctypeslib.ndpointer(np.float32, flags="C")
        u8p = np.ctypeslib.ndpointer(np.uint8, flags="C")
        u32p = np.ctypeslib.ndpointer(np.uint32, flags="C")
        u64p = np.ctypeslib.ndpointer(np.uint64, flags="C")
        L.ppo_surface_distance.argtypes = [f32p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_float, f32p, C.c_int]
        L.ppo_surface_distance.restype = C.c_int
        L.ppo_spatstat.argtypes = [f32p, u8p, C.c_void_p, C.c_uint64, C.c_float, C.c_float, C.c_float,
                                   C.c_uint32, C.c_void_p, C.c_int, C.c_int, u32p, u32p, C.c_void_p,
                                   C.c_int, u64p, C.c_uint64, C.c_void_p, C.c_uint64, C.c_void_p]
        L.ppo_spatstat.restype = C.c_int
        L.ppo_neighbors.argtypes = [f32p, C.c_uint64, C.c_uint64, C.c_float, u64p, f32p, C.c_uint64,
                                    C.POINTER(C.c_uint64)]
        L.ppo_neighbors.restype = C.c_int
        L.ppo_category.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float]
        L.ppo_category.restype = C.c_int
        L.ppo_voxelize.argtypes = [f32p, C.c_uint64, C.c_float, C.c_float, C.POINTER(C.c_uint64),
                                   C.POINTER(C.c_float), u64p]
        L.ppo_voxelize.restype = C.c_int
        L.ppo_npcorr.argtypes = [f32p, u8p, f32p, C.c_uint64, C.c_float, C.c_float, C.c_int, u32p, u32p,
                                 C.c_uint32, u32p, C.c_uint64, C.POINTER(C.c_uint64)]
        L.ppo_npcorr.restype = C.c_int
        L.ppo_aposteriori.argtypes = [f32p, u8p, f32p, C.c_uint64, C.c_float, C.c_float, C.c_float, C.c_uint32,
                                      C.c_int, u64p, C.c_uint64, u64p]
        L.ppo_aposteriori.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def nbins(rmin: float, rincr: float, rmax: float) -> int:
    """Bin count of a reference histogram built from float settings."""
    s, w, e = float(np.float32(rmin)), float(np.float32(rincr)), float(np.float32(rmax))
    return int((e - s) / w) if w > 1e-6 else 0


def type_masks(sets, words: int = 8) -> np.ndarray:
    """List of type-id collections -> (len, 8) uint32 bit masks."""
    m = np.zeros((len(sets), words), dtype=np.uint32)
    for i, s in enumerate(sets):
        for t in s:
            m[i, t >> 5] |= np.uint32(1 << (t & 31))
    return m


def surface_distance(xyz, tri, rprime, nthreads=0):
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    tri = np.ascontiguousarray(tri, dtype=np.float32).reshape(-1, 9)
    out = np.empty(xyz.shape[0], dtype=np.float32)
    rc = lib().ppo_surface_distance(xyz.reshape(-1), xyz.shape[0], _ptr(tri), tri.shape[0],
                                    np.float32(rprime), out, nthreads)
    if rc:
        raise RuntimeError(f"ppo_surface_distance failed ({rc})")
    return out


def spatstat(xyz, labels, ion2surf, rmin, rincr, rmax, analyses, trg, env, k_list=(),
             centre_mask=None, nthreads=0, cntnb_len=4096):
    """Returns dict(bins=uint64 array in pp_fetch layout, cntnb=(ntasks, L),
    centres, discarded, pairs, nbins)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    labels = np.ascontiguousarray(labels, dtype=np.uint8)
    surf = None if ion2surf is None else np.ascontiguousarray(ion2surf, dtype=np.float32)
    cm = None if centre_mask is None else np.ascontiguousarray(centre_mask, dtype=np.uint8)
    tm, em = type_masks(trg), type_masks(env)
    nt = len(trg)
    ks = np.ascontiguousarray(np.asarray(k_list, dtype=np.uint32))
    nk = len(ks) if analyses & MKNN else 0
    nb = nbins(rmin, rincr, rmax)
    ngroups = sum(1 for a in (RDF, NN1, RIPK) if analyses & a) + nk
    out = np.zeros(max(1, ngroups * nt * (nb + 2)), dtype=np.uint64)
    cnt = np.zeros(max(1, nt * cntnb_len), dtype=np.uint64)
    stats = np.zeros(5, dtype=np.uint64)
    rc = lib().ppo_spatstat(xyz.reshape(-1), labels, _ptr(surf), xyz.shape[0], np.float32(rmin),
                            np.float32(rincr), np.float32(rmax), analyses, _ptr(ks), nk, nt,
                            tm.reshape(-1), em.reshape(-1), _ptr(cm), nthreads, out, out.size,
                            _ptr(cnt), cntnb_len if analyses & CNTNB else 0, _ptr(stats))
    if rc:
        raise RuntimeError(f"ppo_spatstat failed ({rc})")
    return dict(bins=out[: ngroups * nt * (nb + 2)], cntnb=cnt[: nt * cntnb_len].reshape(nt, cntnb_len),
                centres=int(stats[0]), discarded=int(stats[1]), pairs=int(stats[2]), nbins=nb,
                build_s=float(stats[3]) * 1e-9, compute_s=float(stats[4]) * 1e-9)


def neighbors(xyz, centre, R):
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    cap = 1 << 16
    ids = np.zeros(cap, dtype=np.uint64)
    d2 = np.zeros(cap, dtype=np.float32)
    cnt = C.c_uint64(0)
    rc = lib().ppo_neighbors(xyz.reshape(-1), xyz.shape[0], centre, np.float32(R), ids, d2, cap, C.byref(cnt))
    if rc:
        raise RuntimeError("ppo_neighbors failed")
    n = min(cnt.value, cap)
    return ids[:n].copy(), d2[:n].copy()


def category(rmin, rincr, rmax, x):
    return lib().ppo_category(np.float32(rmin), np.float32(rincr), np.float32(rmax), np.float32(x))


def voxelize(xyz, w_min=1.0, w_max=1.0):
    """NumberOfIonsInside, VolumeInside and voxel counts of the occupancy grid."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    nin, vol = C.c_uint64(), C.c_float()
    bins = np.zeros(6, dtype=np.uint64)
    rc = lib().ppo_voxelize(xyz.reshape(-1), xyz.shape[0], np.float32(w_min), np.float32(w_max), C.byref(nin),
                            C.byref(vol), bins)
    if rc:
        raise RuntimeError(f"ppo_voxelize failed ({rc})")
    return dict(nions_inside=nin.value, volume_inside=np.float32(vol.value), vacuum=int(bins[0]),
                surface=int(bins[1]), inside=int(bins[2]), nx=int(bins[3]), ny=int(bins[4]), nz=int(bins[5]))


def npcorr(xyz, labels, ion2surf, rincr, rmax, trg, env, order):
    """n-point correlation counts: (ntasks, edge, edge, edge) uint32, [z][y][x]."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    labels = np.ascontiguousarray(labels, dtype=np.uint8)
    surf = np.ascontiguousarray(ion2surf, dtype=np.float32)
    tm, em = type_masks(trg), type_masks(env)
    half = int(np.ceil(np.float32(rmax) / np.float32(rincr)) + 1)
    edge = 1 + 2 * half
    out = np.zeros(len(trg) * edge ** 3, dtype=np.uint32)
    e = C.c_uint64()
    rc = lib().ppo_npcorr(xyz.reshape(-1), labels, surf, xyz.shape[0], np.float32(rincr), np.float32(rmax), len(trg),
                          tm.reshape(-1), em.reshape(-1), order, out, out.size, C.byref(e))
    if rc:
        raise RuntimeError(f"ppo_npcorr failed ({rc})")
    return out.reshape(len(trg), edge, edge, edge)


def aposteriori(xyz, clustered, ion2surf, rmin, rincr, rmax, analyses, guard_mode=0):
    """Statistics after clustering: ({"rdf"|"1nn"|"ripk": (H,) uint64}, stats),
    stats = (centres, guard ions, centres without an unclustered neighbour).
    guard_mode 0: every unclustered ion within R of a clustered one is guard;
    1: the reference's guard loop as written (positions = input order)."""
    xyz = np.ascontiguousarray(xyz, dtype=np.float32)
    clus = np.ascontiguousarray(clustered, dtype=np.uint8)
    surf = np.ascontiguousarray(ion2surf, dtype=np.float32)
    H = nbins(rmin, rincr, rmax) + 2
    names = [nm for bit, nm in ((RDF, "rdf"), (NN1, "1nn"), (RIPK, "ripk")) if analyses & bit]
    out = np.zeros(max(1, len(names)) * H, dtype=np.uint64)
    st = np.zeros(3, dtype=np.uint64)
    rc = lib().ppo_aposteriori(xyz.reshape(-1), clus, surf, xyz.shape[0], np.float32(rmin), np.float32(rincr),
                               np.float32(rmax), analyses, guard_mode, out, out.size, st)
    if rc:
        raise RuntimeError(f"ppo_aposteriori failed ({rc})")
    return {nm: out[i * H:(i + 1) * H].copy() for i, nm in enumerate(names)}, tuple(int(v) for v in st)
