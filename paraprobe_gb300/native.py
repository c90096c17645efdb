"""ctypes binding of libparaprobe_gb300.so (the C ABI in include/paraprobe_gb300.h).

This is plumbing for tests, the benchmark and Python users; the product is the
C ABI itself.  Loading fails loudly when the library has not been built --
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libparaprobe_gb300.so")

PP_RDF, PP_1NN, PP_RIPK, PP_MKNN, PP_NPCORR, PP_CNTNB = 1, 2, 4, 8, 16, 32
PP_OK, PP_ERR_INVALID, PP_ERR_CUDA, PP_ERR_NOMEM, PP_ERR_UNSUPPORTED = 0, -1, -2, -3, -4
PP_ERR_STATE, PP_ERR_OVERFLOW, PP_ERR_DEVICE, PP_ERR_IO = -5, -6, -7, -8
PP_TILE_LANES = 0x100  # tile code (cells << 16) | PP_TILE_LANES: centre-per-lane scan of RDF/RIPK passes

# every symbol include/paraprobe_gb300.h declares
EXPORTS = (
    "pp_create", "pp_destroy", "pp_strerror", "pp_last_error", "pp_cloud_upload", "pp_cloud_upload_device",
    "pp_cloud_upload_pos", "pp_cloud_free", "pp_cloud_labels", "pp_hull_upload", "pp_surfdist_upload",
    "pp_surfdist_fetch", "pp_tasks_set", "pp_hist_params", "pp_run", "pp_fetch", "pp_fetch_cntnb",
    "pp_result_size", "pp_run_stats", "pp_run_batched", "pp_batched_count", "pp_fetch_batched",
    "pp_batched_stats", "pp_neighbors", "pp_shuffle_labels", "pp_device_info", "pp_kernel_launches",
    "pp_last_kernel_ms", "pp_autotune", "pp_cloud_tuning", "pp_set_option", "pp_cloud_prepare",
    "pp_server_create", "pp_server_submit", "pp_server_wait", "pp_server_stats", "pp_server_destroy",
    "pp_fp64_audit", "pp_surfdist_noalloc", "pp_batched_graph", "pp_cloud_inside", "pp_fetch_npcorr",
    "pp_run_aposteriori", "pp_last_kernel", "pp_run_tests", "pp_run_masked", "pp_server_passes",
)

_lib = None


class PPError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{msg} (code {code})")
        self.code = code


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run paraprobe_gb300.build.build() first")
    L = C.CDLL(LIB_PATH)
    vp, u64, i32, u32, f32 = C.c_void_p, C.c_uint64, C.c_int, C.c_uint32, C.c_float
    sig = {
        "pp_create": ([C.POINTER(vp), i32], i32),
        "pp_destroy": ([vp], None),
        "pp_strerror": ([i32], C.c_char_p),
        "pp_last_error": ([vp], C.c_char_p),
        "pp_cloud_upload": ([vp, vp, vp, vp, u64, C.POINTER(i32)], i32),
        "pp_cloud_upload_device": ([vp, vp, vp, u64, C.POINTER(i32), vp], i32),
        "pp_cloud_upload_pos": ([vp, vp, u64, vp, vp, vp, i32, C.POINTER(i32)], i32),
        "pp_cloud_free": ([vp, i32], i32),
        "pp_cloud_labels": ([vp, i32, vp, u64], i32),
        "pp_hull_upload": ([vp, i32, vp, u64, f32], i32),
        "pp_surfdist_upload": ([vp, i32, vp], i32),
        "pp_surfdist_fetch": ([vp, i32, vp, u64], i32),
        "pp_tasks_set": ([vp, vp, vp, i32], i32),
        "pp_hist_params": ([vp, f32, f32, f32], i32),
        "pp_run": ([vp, i32, u32, vp, i32, vp, vp], i32),
        "pp_run_masked": ([vp, i32, u32, vp, i32, vp, vp, vp], i32),
        "pp_fetch": ([vp, vp, C.c_size_t], i32),
        "pp_fetch_cntnb": ([vp, vp, C.c_size_t, C.POINTER(u64)], i32),
        "pp_result_size": ([vp, C.POINTER(u64), C.POINTER(u64)], i32),
        "pp_run_stats": ([vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)], i32),
        "pp_run_batched": ([vp, i32, u32, vp, i32, i32, vp, i32, vp, i32, vp], i32),
        "pp_batched_count": ([vp, C.POINTER(i32)], i32),
        "pp_fetch_batched": ([vp, i32, vp, C.c_size_t], i32),
        "pp_batched_stats": ([vp, i32, C.POINTER(u64), C.POINTER(u64)], i32),
        "pp_neighbors": ([vp, i32, u64, f32, vp, vp, u64, C.POINTER(u64)], i32),
        "pp_shuffle_labels": ([vp, u64, u64, vp], i32),
        "pp_device_info": ([vp, C.POINTER(i32), C.POINTER(i32)], i32),
        "pp_kernel_launches": ([C.POINTER(u64)], i32),
        "pp_last_kernel_ms": ([vp, C.POINTER(f32)], i32),
        "pp_autotune": ([vp, i32, u32, vp, i32, u32, C.POINTER(f32), C.POINTER(u32)], i32),
        "pp_cloud_tuning": ([vp, i32, f32, u32], i32),
        "pp_set_option": ([vp, C.c_char_p, i32], i32),
        "pp_cloud_prepare": ([vp, i32, f32, f32], i32),
        "pp_server_create": ([vp, i32, u64, C.POINTER(vp)], i32),
        "pp_server_submit": ([vp, i32, u32, f32, f32, f32, vp, vp, i32, vp, i32, C.POINTER(u64)], i32),
        "pp_server_wait": ([vp, u64, vp, C.c_size_t, C.POINTER(u64), C.POINTER(u64), C.POINTER(C.c_double)], i32),
        "pp_server_stats": ([vp, C.POINTER(C.c_double)], i32),
        "pp_server_destroy": ([vp], None),
        "pp_server_passes": ([vp, C.POINTER(u64), C.POINTER(u64)], i32),
        "pp_fp64_audit": ([vp, i32, u32, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(u64),
                           C.POINTER(u64), C.POINTER(u64), vp, vp, u64, C.POINTER(u64)], i32),
        "pp_surfdist_noalloc": ([vp, u64, vp, u64, f32, vp, vp, C.c_char_p, C.c_size_t], i32),
        "pp_batched_graph": ([vp, C.POINTER(u64), C.POINTER(u64), C.POINTER(u64)], i32),
        "pp_cloud_inside": ([vp, i32, f32, f32, C.POINTER(u64), C.POINTER(f32), vp], i32),
        "pp_fetch_npcorr": ([vp, vp, u64, C.POINTER(u64)], i32),
        "pp_run_aposteriori": ([vp, i32, vp, u32, vp], i32),
        "pp_last_kernel": ([vp, C.POINTER(C.c_char_p)], i32),
        "pp_run_tests": ([vp, C.POINTER(u64)], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def type_masks(sets) -> np.ndarray:
    """List of type-id collections -> (len, 8) uint32 masks (256 type bits)."""
    m = np.zeros((len(sets), 8), dtype=np.uint32)
    for i, s in enumerate(sets):
        for t in s:
            m[i, int(t) >> 5] |= np.uint32(1 << (int(t) & 31))
    return m


def kernel_launches() -> int:
    n = C.c_uint64()
    load().pp_kernel_launches(C.byref(n))
    return n.value


def shuffle_labels(labels, seed):
    lab = np.ascontiguousarray(labels, dtype=np.uint8)
    out = np.empty_like(lab)
    rc = load().pp_shuffle_labels(_p(lab), lab.size, seed, _p(out))
    if rc:
        raise PPError(rc, "pp_shuffle_labels failed")
    return out


class Context:
    """One pp_ctx on one CUDA device."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = C.c_void_p()
        rc = self.L.pp_create(C.byref(h), device)
        if rc:
            raise PPError(rc, "pp_create failed: " + self.L.pp_strerror(rc).decode())
        self.h = h

    def close(self):
        if self.h:
            self.L.pp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc, what):
        if rc:
            msg = self.L.pp_last_error(self.h).decode(errors="replace")
            raise PPError(rc, f"{what}: {self.L.pp_strerror(rc).decode()}: {msg}")

    def run_tests(self) -> int:
        """Candidate distance tests of the last run."""
        t = C.c_uint64()
        self._ck(self.L.pp_run_tests(self.h, C.byref(t)), "pp_run_tests")
        return t.value

    def last_kernel(self) -> str:
        """Name of the stencil kernel the last run took."""
        nm = C.c_char_p()
        self._ck(self.L.pp_last_kernel(self.h, C.byref(nm)), "pp_last_kernel")
        return nm.value.decode()

    def last_kernel_ms(self) -> float:
        ms = C.c_float()
        self._ck(self.L.pp_last_kernel_ms(self.h, C.byref(ms)), "pp_last_kernel_ms")
        return ms.value

    def sm_count(self):
        d, s = C.c_int(), C.c_int()
        self._ck(self.L.pp_device_info(self.h, C.byref(d), C.byref(s)), "pp_device_info")
        return s.value

    # ---- clouds
    def upload(self, xyz, labels, ion_id=None) -> int:
        xyz = np.ascontiguousarray(xyz, dtype=np.float32)
        lab = np.ascontiguousarray(labels, dtype=np.uint8)
        ids = None if ion_id is None else np.ascontiguousarray(ion_id, dtype=np.uint32)
        cid = C.c_int()
        self._ck(self.L.pp_cloud_upload(self.h, _p(xyz), _p(lab), _p(ids), lab.size, C.byref(cid)), "pp_cloud_upload")
        return cid.value

    def upload_device(self, xyz_ptr: int, label_ptr: int, n: int, stream: int = 0) -> int:
        cid = C.c_int()
        self._ck(self.L.pp_cloud_upload_device(self.h, C.c_void_p(xyz_ptr), C.c_void_p(label_ptr), n,
                                               C.byref(cid), C.c_void_p(stream)), "pp_cloud_upload_device")
        return cid.value

    def upload_pos(self, pos_bytes, ranges) -> int:
        """ranges: list of (lo, hi, type) in the order mq2ionname visits them."""
        raw = np.frombuffer(pos_bytes, dtype=np.uint8) if isinstance(pos_bytes, (bytes, bytearray)) else \
            np.ascontiguousarray(pos_bytes).view(np.uint8)
        n = raw.size // 16
        lo = np.ascontiguousarray([r[0] for r in ranges], dtype=np.float32)
        hi = np.ascontiguousarray([r[1] for r in ranges], dtype=np.float32)
        ty = np.ascontiguousarray([r[2] for r in ranges], dtype=np.uint8)
        cid = C.c_int()
        self._ck(self.L.pp_cloud_upload_pos(self.h, _p(raw), n, _p(lo), _p(hi), _p(ty), len(ranges), C.byref(cid)),
                 "pp_cloud_upload_pos")
        return cid.value

    def cloud_labels(self, cloud, n):
        out = np.empty(n, dtype=np.uint8)
        self._ck(self.L.pp_cloud_labels(self.h, cloud, _p(out), n), "pp_cloud_labels")
        return out

    def free(self, cloud):
        self._ck(self.L.pp_cloud_free(self.h, cloud), "pp_cloud_free")

    def hull(self, cloud, tri, carve_radius=2.0):
        tri = np.ascontiguousarray(tri, dtype=np.float32).reshape(-1, 9)
        self._ck(self.L.pp_hull_upload(self.h, cloud, _p(tri), tri.shape[0], carve_radius), "pp_hull_upload")

    def surfdist(self, cloud, d2):
        d2 = np.ascontiguousarray(d2, dtype=np.float32)
        self._ck(self.L.pp_surfdist_upload(self.h, cloud, _p(d2)), "pp_surfdist_upload")

    def surfdist_fetch(self, cloud, n):
        out = np.empty(n, dtype=np.float32)
        self._ck(self.L.pp_surfdist_fetch(self.h, cloud, _p(out), n), "pp_surfdist_fetch")
        return out

    # ---- query
    def tasks(self, trg, env):
        tm, em = type_masks(trg), type_masks(env)
        self._ck(self.L.pp_tasks_set(self.h, _p(tm), _p(em), len(trg)), "pp_tasks_set")
        self.ntasks = len(trg)

    def hist(self, rmin, rincr, rmax):
        self._ck(self.L.pp_hist_params(self.h, rmin, rincr, rmax), "pp_hist_params")

    def run(self, cloud, flags, k_list=(), label_perm=None, stream=0, centre_mask=None):
        """One pass; centre_mask (n bytes, input order) restricts the centres further."""
        ks = np.ascontiguousarray(np.asarray(k_list, dtype=np.uint32))
        perm = None if label_perm is None else np.ascontiguousarray(label_perm, dtype=np.uint32)
        if centre_mask is None:
            self._ck(self.L.pp_run(self.h, cloud, flags, _p(ks) if ks.size else None, ks.size, _p(perm),
                                   C.c_void_p(stream)), "pp_run")
        else:
            cm = np.ascontiguousarray(centre_mask, dtype=np.uint8)
            self._ck(self.L.pp_run_masked(self.h, cloud, flags, _p(ks) if ks.size else None, ks.size, _p(perm),
                                          _p(cm), C.c_void_p(stream)), "pp_run_masked")

    def autotune(self, cloud, flags, k_list=(), sample=0):
        ks = np.ascontiguousarray(np.asarray(k_list, dtype=np.uint32))
        r, t = C.c_float(), C.c_uint32()
        self._ck(self.L.pp_autotune(self.h, cloud, flags, _p(ks) if ks.size else None, ks.size, sample,
                                    C.byref(r), C.byref(t)), "pp_autotune")
        return r.value, t.value

    def fp64_audit(self, cloud, max_centres=0, cap=4096):
        """FP64 recomputation of the current tasks' distances and bins."""
        ma, mr = C.c_double(), C.c_double()
        pairs, bd, sd, nl = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        ids = np.zeros((max(cap, 1), 2), dtype=np.uint64)
        dd = np.zeros((max(cap, 1), 2), dtype=np.float64)
        self._ck(self.L.pp_fp64_audit(self.h, cloud, max_centres, C.byref(ma), C.byref(mr), C.byref(pairs),
                                      C.byref(bd), C.byref(sd), _p(ids), _p(dd), cap, C.byref(nl)), "pp_fp64_audit")
        return dict(max_abs_err=ma.value, max_rel_err=mr.value, pairs=pairs.value, bin_disagreements=bd.value,
                    set_disagreements=sd.value, listed_ids=ids[: nl.value], listed_d=dd[: nl.value])

    def prepare(self, cloud, r_lo, r_hi):
        self._ck(self.L.pp_cloud_prepare(self.h, cloud, r_lo, r_hi), "pp_cloud_prepare")

    def set_option(self, name, value):
        self._ck(self.L.pp_set_option(self.h, name.encode(), int(value)), "pp_set_option")

    def tuning(self, cloud, cell_ratio, tile):
        self._ck(self.L.pp_cloud_tuning(self.h, cloud, cell_ratio, tile), "pp_cloud_tuning")

    def result_size(self):
        t, nb = C.c_uint64(), C.c_uint64()
        self._ck(self.L.pp_result_size(self.h, C.byref(t), C.byref(nb)), "pp_result_size")
        return t.value, nb.value

    def fetch(self):
        total, _ = self.result_size()
        out = np.zeros(max(total, 1), dtype=np.uint64)
        self._ck(self.L.pp_fetch(self.h, _p(out), out.size), "pp_fetch")
        return out[:total]

    def fetch_cntnb(self):
        ln = C.c_uint64()
        self._ck(self.L.pp_fetch_cntnb(self.h, None, 0, C.byref(ln)), "pp_fetch_cntnb")
        out = np.zeros(max(ln.value * self.ntasks, 1), dtype=np.uint64)
        self._ck(self.L.pp_fetch_cntnb(self.h, _p(out), out.size, C.byref(ln)), "pp_fetch_cntnb")
        return out[: ln.value * self.ntasks].reshape(self.ntasks, ln.value)

    def stats(self):
        c, d, p = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._ck(self.L.pp_run_stats(self.h, C.byref(c), C.byref(d), C.byref(p)), "pp_run_stats")
        return dict(centres=c.value, discarded=d.value, pairs=p.value)

    def run_batched(self, cloud, flags, k_list=(), include_original=True, label_sets=None, rois=None, stream=0,
                    nsets=None):
        """label_sets: (nsets, n) uint8 array, or a device pointer (int) with nsets given."""
        ks = np.ascontiguousarray(np.asarray(k_list, dtype=np.uint32))
        if isinstance(label_sets, int):
            lp, nls = C.c_void_p(label_sets), int(nsets)
        else:
            ls = None if label_sets is None else np.ascontiguousarray(label_sets, dtype=np.uint8)
            nls = 0 if ls is None else (ls.shape[0] if ls.ndim == 2 else 1)
            lp = _p(ls)
        rr = None if rois is None else np.ascontiguousarray(rois, dtype=np.float32).reshape(-1, 4)
        nr = 0 if rr is None else rr.shape[0]
        self._ck(self.L.pp_run_batched(self.h, cloud, flags, _p(ks) if ks.size else None, ks.size,
                                       1 if include_original else 0, lp, nls, _p(rr), nr, C.c_void_p(stream)),
                 "pp_run_batched")

    def batched_count(self):
        n = C.c_int()
        self._ck(self.L.pp_batched_count(self.h, C.byref(n)), "pp_batched_count")
        return n.value

    def fetch_batched(self, r):
        total, _ = self.result_size()
        out = np.zeros(max(total, 1), dtype=np.uint64)
        self._ck(self.L.pp_fetch_batched(self.h, r, _p(out), out.size), "pp_fetch_batched")
        return out[:total]

    def batched_stats(self, r):
        c, p = C.c_uint64(), C.c_uint64()
        self._ck(self.L.pp_batched_stats(self.h, r, C.byref(c), C.byref(p)), "pp_batched_stats")
        return dict(centres=c.value, pairs=p.value)

    def inside(self, cloud, bin_width_min=1.0, bin_width_max=1.0):
        """NumberOfIonsInside, VolumeInside and the voxel counts of the occupancy grid."""
        nin, vol = C.c_uint64(), C.c_float()
        vox = np.zeros(6, dtype=np.uint64)
        self._ck(self.L.pp_cloud_inside(self.h, cloud, bin_width_min, bin_width_max, C.byref(nin), C.byref(vol),
                                        _p(vox)), "pp_cloud_inside")
        return dict(nions_inside=nin.value, volume_inside=np.float32(vol.value), vacuum=int(vox[0]),
                    surface=int(vox[1]), inside=int(vox[2]), nx=int(vox[3]), ny=int(vox[4]), nz=int(vox[5]))

    def run_aposteriori(self, cloud, clustered, flags, stream=0):
        """Statistics after clustering; clustered: per ion in input order, nonzero = in a cluster.
        The result (one task) is read with fetch()."""
        cf = np.ascontiguousarray(clustered, dtype=np.uint8)
        self._ck(self.L.pp_run_aposteriori(self.h, cloud, _p(cf), flags, C.c_void_p(stream)), "pp_run_aposteriori")

    def fetch_npcorr(self):
        """n-point correlation counts of the last pass: (ntasks, edge, edge, edge) uint32."""
        e = C.c_uint64()
        self._ck(self.L.pp_fetch_npcorr(self.h, None, 0, C.byref(e)), "pp_fetch_npcorr")
        edge = e.value
        ntasks = self.ntasks
        out = np.zeros(max(ntasks * edge ** 3, 1), dtype=np.uint32)
        self._ck(self.L.pp_fetch_npcorr(self.h, _p(out), out.size, C.byref(e)), "pp_fetch_npcorr")
        return out[: ntasks * edge ** 3].reshape(ntasks, edge, edge, edge)

    def batched_graph(self):
        nodes, caps, launches = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._ck(self.L.pp_batched_graph(self.h, C.byref(nodes), C.byref(caps), C.byref(launches)),
                 "pp_batched_graph")
        return dict(nodes=nodes.value, captures=caps.value, launches=launches.value)

    def neighbors(self, cloud, ion, r):
        cnt = C.c_uint64()
        self._ck(self.L.pp_neighbors(self.h, cloud, ion, r, None, None, 0, C.byref(cnt)), "pp_neighbors")
        ids = np.zeros(max(cnt.value, 1), dtype=np.uint64)
        d2 = np.zeros(max(cnt.value, 1), dtype=np.float32)
        self._ck(self.L.pp_neighbors(self.h, cloud, ion, r, _p(ids), _p(d2), cnt.value, C.byref(cnt)), "pp_neighbors")
        return ids[: cnt.value], d2[: cnt.value]


class Server:
    """Continuous-batching query server over the clouds of a Context."""

    def __init__(self, ctx: Context, slots: int = 4, budget_bytes: int = 8 << 30):
        self.ctx = ctx
        self.L = ctx.L
        h = C.c_void_p()
        rc = self.L.pp_server_create(ctx.h, slots, budget_bytes, C.byref(h))
        if rc:
            raise PPError(rc, "pp_server_create failed: " + self.L.pp_last_error(ctx.h).decode())
        self.h = h

    def submit(self, cloud, flags, hist, trg, env, k_list=()):
        tm, em = type_masks(trg), type_masks(env)
        ks = np.ascontiguousarray(np.asarray(k_list, dtype=np.uint32))
        t = C.c_uint64()
        rc = self.L.pp_server_submit(self.h, cloud, flags, hist[0], hist[1], hist[2], _p(tm), _p(em), len(trg),
                                     _p(ks) if ks.size else None, ks.size, C.byref(t))
        if rc:
            raise PPError(rc, "pp_server_submit rejected the query")
        return t.value

    def wait(self, ticket, cap=1 << 22):
        out = np.zeros(cap, dtype=np.uint64)
        ln, pairs, lat = C.c_uint64(), C.c_uint64(), C.c_double()
        rc = self.L.pp_server_wait(self.h, ticket, _p(out), cap, C.byref(ln), C.byref(pairs), C.byref(lat))
        if rc:
            raise PPError(rc, "query failed")
        return out[: ln.value].copy(), pairs.value, lat.value

    def stats(self):
        st = (C.c_double * 8)()
        self.L.pp_server_stats(self.h, st)
        keys = ("submitted", "admitted", "rejected", "completed", "in_flight", "p50_ms", "p99_ms", "pairs")
        return dict(zip(keys, list(st)))

    def passes(self):
        """(merged passes run, queries they took)."""
        p, q = C.c_uint64(), C.c_uint64()
        self.L.pp_server_passes(self.h, C.byref(p), C.byref(q))
        return p.value, q.value

    def close(self):
        if self.h:
            self.L.pp_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
