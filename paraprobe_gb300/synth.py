"""Synthetic atom-probe specimens and PARAPROBE input files.

Generates labelled 3-D ion clouds in the two specimen geometries used to
exercise the spatial-statistics path -- a cylinder and a truncated cone
("tip") -- with uniform Poisson matrix ions, optional Gaussian solute
clusters, and iid minority species.  Writes the inputs PARAPROBE reads for
that path: a big-endian POS file (x, y, z, m/q as float32; format of
src/PARAPROBE_EPOSEndianness.h:40-79), an RRNG range file (read by
src/PARAPROBE_PeriodicTable.cpp:324-420), a closed triangle hull as a naive
VTK polydata file (read by src/PARAPROBE_SolverHdl.cpp:2029-2118) and the XML
settings keys of the descriptive-statistics task
(src/PARAPROBE_Settings.cpp:181-503).

All randomness comes from numpy's PCG64 with an explicit seed, so a given
(seed, parameters) pair always produces the same specimen.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# Element names used for species 0..7.  Every name has two characters so that
# the RRNG reader's single-character special case never applies.
ELEMENTS = ("Al", "Sc", "Zr", "Si", "Mg", "Fe", "Cu", "Ti")


@dataclass
class Specimen:
    """An ion cloud plus the hull that bounds it."""
    xyz: np.ndarray            # (n, 3) float32
    species: np.ndarray        # (n,) uint8, 0-based species index
    hull: np.ndarray           # (t, 9) float32 triangles
    nspecies: int
    meta: dict = field(default_factory=dict)

    @property
    def labels(self) -> np.ndarray:
        """PARAPROBE type ids: species + 1 (type 0 is 'Unknown')."""
        return (self.species.astype(np.uint8) + 1).astype(np.uint8)


# --------------------------------------------------------------- geometry
def cylinder_volume(radius: float, height: float) -> float:
    return math.pi * radius * radius * height


def cone_radius_top(r_apex: float, half_angle_deg: float, length: float) -> float:
    return r_apex + length * math.tan(math.radians(half_angle_deg))


def cone_volume(r_apex: float, half_angle_deg: float, length: float) -> float:
    r1 = cone_radius_top(r_apex, half_angle_deg, length)
    return math.pi * length * (r_apex * r_apex + r_apex * r1 + r1 * r1) / 3.0


def cone_length_for(n: int, rho: float, r_apex: float, half_angle_deg: float) -> float:
    """Length of a truncated cone that holds n ions at density rho."""
    lo, hi = 0.0, 1.0
    while cone_volume(r_apex, half_angle_deg, hi) * rho < n:
        hi *= 2.0
    for _ in range(100):
        mid = 0.5 * (lo + hi)
        if cone_volume(r_apex, half_angle_deg, mid) * rho < n:
            lo = mid
        else:
            hi = mid
    return hi


def _uniform_in_cylinder(rng, n, radius, height):
    r = radius * np.sqrt(rng.random(n))
    phi = 2.0 * math.pi * rng.random(n)
    z = height * rng.random(n)
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def _uniform_in_cone(rng, n, r_apex, half_angle_deg, length):
    tn = math.tan(math.radians(half_angle_deg))
    r1 = r_apex + length * tn
    # z density is proportional to r(z)^2; invert the cubic CDF exactly.
    u = rng.random(n)
    if tn > 0:
        c = r_apex ** 3 + u * (r1 ** 3 - r_apex ** 3)
        z = (np.cbrt(c) - r_apex) / tn
    else:
        z = u * length
    rz = r_apex + z * tn
    r = rz * np.sqrt(rng.random(n))
    phi = 2.0 * math.pi * rng.random(n)
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def _inside_cone(p, r_apex, half_angle_deg, length):
    tn = math.tan(math.radians(half_angle_deg))
    z = p[:, 2]
    rz = r_apex + z * tn
    return (z >= 0) & (z <= length) & (p[:, 0] ** 2 + p[:, 1] ** 2 <= rz * rz)


# ------------------------------------------------------------- generators
def cylinder_specimen(n: int = 1_000_000, radius: float = 10.0, height: float = 63.66,
                      fractions=(0.90, 0.08, 0.02), seed: int = 20261204,
                      nseg: int = 512, stack: float = 2.0) -> Specimen:
    """Uniform Poisson ions (fixed n) in a cylinder with iid species labels."""
    rng = np.random.Generator(np.random.PCG64(seed))
    xyz = _uniform_in_cylinder(rng, n, radius, height).astype(np.float32)
    p = np.asarray(fractions, dtype=np.float64)
    species = rng.choice(len(p), size=n, p=p / p.sum()).astype(np.uint8)
    hull = cylinder_hull(radius, height, nseg=nseg, stack=stack)
    return Specimen(xyz, species, hull, len(p),
                    dict(kind="cylinder", n=n, radius=radius, height=height,
                         fractions=list(fractions), seed=seed))


def cone_specimen(n: int = 20_000_000, r_apex: float = 30.0, half_angle_deg: float = 10.0,
                  length: float = 200.0, n_clusters: int = 2000, sigma: float = 1.5,
                  members: int = 50, cluster_p=(0.7, 0.3), iid=(0.02, 0.01, 0.005),
                  nspecies: int = 6, seed: int = 20261205, nseg: int = 512,
                  stack: float = 2.0) -> Specimen:
    """Clustered specimen in a truncated cone.

    Matrix ions are uniform Poisson (species 0).  n_clusters centres are
    uniform inside the cone; each carries `members` ions displaced by an
    isotropic Gaussian of width sigma, labelled species 1 or 2 with
    probabilities cluster_p (members falling outside the cone are redrawn).
    Matrix ions become species 3, 4, ... with the iid probabilities `iid`;
    with nspecies > 3 + len(iid) the remaining species share the last iid
    probability.  Total ion count is exactly n.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    ncl = min(n, n_clusters * members)
    centres = _uniform_in_cone(rng, n_clusters, r_apex, half_angle_deg, length)
    pts = []
    need = ncl
    while need > 0:
        who = rng.integers(0, n_clusters, size=need)
        cand = centres[who] + sigma * rng.standard_normal((need, 3))
        cand = cand[_inside_cone(cand, r_apex, half_angle_deg, length)]
        pts.append(cand)
        need -= len(cand)
    clus = np.concatenate(pts)[:ncl] if ncl else np.zeros((0, 3))
    csp = np.where(rng.random(ncl) < cluster_p[0], 1, 2).astype(np.uint8)
    mat = _uniform_in_cone(rng, n - ncl, r_apex, half_angle_deg, length)
    extra = list(iid)
    while 3 + len(extra) < nspecies:
        extra.append(extra[-1] if extra else 0.0)
    extra = extra[: max(0, nspecies - 3)]
    probs = np.array([1.0 - sum(extra)] + extra)
    msp = rng.choice(len(probs), size=n - ncl, p=probs).astype(np.uint8)
    msp = np.where(msp == 0, 0, msp + 2).astype(np.uint8)
    xyz = np.concatenate([mat, clus]).astype(np.float32)
    species = np.concatenate([msp, csp])
    order = rng.permutation(n)
    hull = cone_hull(r_apex, half_angle_deg, length, nseg=nseg, stack=stack)
    return Specimen(xyz[order], species[order], hull, nspecies,
                    dict(kind="cone", n=n, r_apex=r_apex, half_angle_deg=half_angle_deg,
                         length=length, n_clusters=n_clusters, sigma=sigma, members=members,
                         cluster_p=list(cluster_p), iid=extra, seed=seed))


# ------------------------------------------------------------------ hulls
def _frustum_hull(r0: float, r1: float, length: float, nseg: int, stack: float) -> np.ndarray:
    """Closed triangulated frustum (side + two end caps), float32 (t, 9)."""
    nst = max(1, int(math.ceil(length / stack)))
    phi = 2.0 * math.pi * np.arange(nseg) / nseg
    c, s = np.cos(phi), np.sin(phi)
    tris = []
    for k in range(nst):
        z0, z1 = length * k / nst, length * (k + 1) / nst
        ra, rb = r0 + (r1 - r0) * k / nst, r0 + (r1 - r0) * (k + 1) / nst
        a = np.stack([ra * c, ra * s, np.full(nseg, z0)], 1)
        b = np.stack([rb * c, rb * s, np.full(nseg, z1)], 1)
        a2, b2 = np.roll(a, -1, 0), np.roll(b, -1, 0)
        tris.append(np.concatenate([a, a2, b], 1))
        tris.append(np.concatenate([a2, b2, b], 1))
    for z, r in ((0.0, r0), (length, r1)):
        ring = np.stack([r * c, r * s, np.full(nseg, z)], 1)
        ctr = np.tile(np.array([[0.0, 0.0, z]]), (nseg, 1))
        tris.append(np.concatenate([ctr, ring, np.roll(ring, -1, 0)], 1))
    return np.concatenate(tris).astype(np.float32)


def cylinder_hull(radius: float, height: float, nseg: int = 512, stack: float = 2.0) -> np.ndarray:
    return _frustum_hull(radius, radius, height, nseg, stack)


def cone_hull(r_apex: float, half_angle_deg: float, length: float, nseg: int = 512,
              stack: float = 2.0) -> np.ndarray:
    return _frustum_hull(r_apex, cone_radius_top(r_apex, half_angle_deg, length), length, nseg, stack)


# ---------------------------------------------------------------- writers
def species_windows(nspecies: int):
    """Distinct m/q windows, one per species: [10 + 5 s, 10 + 5 s + 1]."""
    return [(10.0 + 5.0 * s, 11.0 + 5.0 * s) for s in range(nspecies)]


def species_mq(species: np.ndarray, seed: int = 7) -> np.ndarray:
    """An m/q value inside each ion's species window (never on an edge)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lo = 10.0 + 5.0 * species.astype(np.float64)
    return (lo + 0.1 + 0.8 * rng.random(species.shape[0])).astype(np.float32)


def write_pos(path: str, xyz: np.ndarray, mq: np.ndarray) -> None:
    rec = np.empty((xyz.shape[0], 4), dtype=">f4")
    rec[:, :3] = xyz
    rec[:, 3] = mq
    rec.tofile(path)


def write_epos(path: str, xyz: np.ndarray, mq: np.ndarray, seed: int = 11) -> None:
    """EPOS file: 44-byte big-endian records, nine floats (x, y, z, m/q, tof,
    Vdc, Vpulse, detx, dety) and two int32 (pulses since last, ions per
    pulse); the detector fields are seeded filler."""
    rng = np.random.default_rng(seed)
    n = xyz.shape[0]
    rec = np.zeros(n, dtype=[("f", ">f4", 9), ("i", ">i4", 2)])
    rec["f"][:, :3] = xyz
    rec["f"][:, 3] = mq
    rec["f"][:, 4:] = rng.uniform(0.0, 1000.0, (n, 5)).astype(np.float32)
    rec["i"][:] = rng.integers(0, 4, (n, 2))
    rec.tofile(path)


def read_pos(path: str):
    rec = np.fromfile(path, dtype=">f4").reshape(-1, 4).astype(np.float32)
    return np.ascontiguousarray(rec[:, :3]), np.ascontiguousarray(rec[:, 3])


def write_rrng(path: str, nspecies: int) -> None:
    lines = ["[Ions]", f"Number={nspecies}"]
    lines += [f"Ion{s + 1}={ELEMENTS[s]}" for s in range(nspecies)]
    lines += ["[Ranges]", f"Number={nspecies}"]
    for s, (lo, hi) in enumerate(species_windows(nspecies)):
        lines.append(f"Range{s + 1}={lo:.4f} {hi:.4f} Vol:0.01661 {ELEMENTS[s]}:1 Color:33FFFF")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def write_vtk(path: str, tri: np.ndarray) -> None:
    """Naive VTK polydata with three unshared points per triangle; values are
    printed with 9 significant digits so that float32 parsing is exact."""
    t = np.asarray(tri, dtype=np.float32).reshape(-1, 3, 3)
    with open(path, "w") as f:
        f.write("# vtk DataFile Version 2.0\nPARAPROBE TipSurface\nASCII\nDATASET POLYDATA\n")
        f.write(f"POINTS {t.shape[0] * 3} double\n")
        pts = t.reshape(-1, 3)
        f.write("".join(f"{x:.9g} {y:.9g} {z:.9g}\n" for x, y, z in pts.tolist()))
        f.write("\n")
        f.write(f"POLYGONS {t.shape[0]} {4 * t.shape[0]}\n")
        f.write("".join(f"3 {3 * i} {3 * i + 1} {3 * i + 2}\n" for i in range(t.shape[0])))
        f.write("\n")


def write_settings_xml(path: str, pos: str, rrng: str, vtk: str | None, analyses: str,
                       tasks: str, rmin: str, rincr: str, rmax: str, mknn: str = "",
                       knn_order: int = 1, label_rnd: int = 0, bin_width=None) -> None:
    """XML with the keys the descriptive-statistics path reads; numbers are
    passed as strings so they reach the float parser exactly as written."""
    surf = "4" if vtk else "0"
    body = [
        "<?xml version=\"1.0\" encoding=\"utf-8\"?>", "<Parameters>",
        "\t<InputFileformat>1</InputFileformat>",
        f"\t<RAWFilenameIn>{pos}</RAWFilenameIn>",
        "\t<AnalysisMode>1</AnalysisMode>",
        "\t<ReconstructionAlgorithm>2</ReconstructionAlgorithm>",
        "\t<IdentifyIonType>1</IdentifyIonType>",
        f"\t<RRNGFilenameIn>{rrng}</RRNGFilenameIn>",
        f"\t<SurfaceReconstructionType>{surf}</SurfaceReconstructionType>",
        f"\t<SurfaceFilenameIn>{vtk or ''}</SurfaceFilenameIn>",
        "\t<AnalysisCrystallographicInfo>0</AnalysisCrystallographicInfo>",
        f"\t<AnalysisSpatDistrType>{analyses}</AnalysisSpatDistrType>",
        "\t<AnalysisClusteringType>0</AnalysisClusteringType>",
        "\t<AnalysisVolumeTessellation>0</AnalysisVolumeTessellation>",
        "\t<DebugComputeDistance>1</DebugComputeDistance>",
        f"\t<DescrStatTasksCode>{tasks}</DescrStatTasksCode>",
        f"\t<SpatStatRadiusMin>{rmin}</SpatStatRadiusMin>",
        f"\t<SpatStatRadiusIncr>{rincr}</SpatStatRadiusIncr>",
        f"\t<SpatStatRadiusMax>{rmax}</SpatStatRadiusMax>",
        f"\t<SpatStatKNNOrder>{knn_order}</SpatStatKNNOrder>",
        f"\t<SpatStatMKNNCode>{mknn}</SpatStatMKNNCode>",
        f"\t<SpatStatAdditionalLabelRandomization>{label_rnd}</SpatStatAdditionalLabelRandomization>",
    ]
    if bin_width is not None:  # (min, incr, max) of the occupancy grid, as strings
        body += [f"\t<AdvIonPruneBinWidthMin>{bin_width[0]}</AdvIonPruneBinWidthMin>",
                 f"\t<AdvIonPruneBinWidthIncr>{bin_width[1]}</AdvIonPruneBinWidthIncr>",
                 f"\t<AdvIonPruneBinWidthMax>{bin_width[2]}</AdvIonPruneBinWidthMax>"]
    body += ["</Parameters>", ""]
    with open(path, "w") as f:
        f.write("\n".join(body))


def write_inputs(spec: Specimen, outdir: str, stem: str, seed_mq: int = 7):
    """POS + RRNG + VTK for a specimen; returns their paths."""
    os.makedirs(outdir, exist_ok=True)
    pos = os.path.join(outdir, stem + ".pos")
    rrng = os.path.join(outdir, stem + ".rrng")
    vtk = os.path.join(outdir, stem + ".vtk")
    write_pos(pos, spec.xyz, species_mq(spec.species, seed_mq))
    write_rrng(rrng, spec.nspecies)
    write_vtk(vtk, spec.hull)
    return pos, rrng, vtk


def all_pairs_tasks(nspecies: int) -> str:
    """'A-A;A-B;...' over every ordered species pair."""
    return ";".join(f"{ELEMENTS[a]}-{ELEMENTS[b]}" for a in range(nspecies) for b in range(nspecies))
