"""Seeded synthetic catalogues in the reference's input formats.

The reference is run on catalogues prepared by its ``Gen_inp_*`` notebooks
(``write_data`` in Gen_inp_Periodic_box.ipynb: ``<prefix>_pos.dat`` with two
columns x y (or ra dec), ``_z.dat`` one column, ``_e.dat`` e1 e2, ``_wt.dat``
weights, ``_jk.dat`` integer region labels, all via ``numpy.savetxt``) and a
positional ``.inp`` file (``inp_gen`` in the same notebook; read by
``data_ini`` initialization.cpp:70-130).  This module generates the benchmark
workloads with those shapes and distributions and writes them in exactly that
format, sorted by z as the notebooks do (``S_dat.sort('z')``) so that
``data_sorted 1`` is valid.

Workloads (sizes as named by the project's benchmark list):
  * ``box_uniform``  - 20,000 uniform points, L=250, wgg, 8 jackknife cubes.
  * ``box_ns``       - Neyman-Scott clustered box (2,000 parents x Poisson(100),
                       sigma=2, L=500), float32 positions, wg+, 64 cubes.
  * ``box_batch``    - 64 uniform sub-boxes (L=200, N log-uniform 1e4..4e5),
                       w++ (+wgg, wg+), 27 cubes each.
  * ``box_ns_large`` - 20M-point Neyman-Scott box (200,000 parents, sigma=3,
                       L=1000), float32, w++, 125 cubes.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

# ---------------------------------------------------------------------------
# parameter set written to .inp (order = initialization.cpp:70-130)
# ---------------------------------------------------------------------------

INP_KEYS = [
    # (key written, attribute, kind)
    ("which_corr", "which_corr", int),
    ("coordinates", "coordinates", int),
    ("estimator", "estimator", int),
    ("data_sorted", "data_sorted", int),
    ("use_comoving", "use_comoving", int),
    ("do_jk", "do_jk", int),
    ("sig_crit", "sig_crit", int),
    ("shape_pos", "shape_pos_file", str),
    ("shape_z", "shape_z_file", str),
    ("shape_e", "shape_e_file", str),
    ("shape_wt", "shape_wt_file", str),
    ("shape_jk", "shape_jk_file", str),
    ("shape_patch", "shape_patch_file", str),
    ("density_pos", "density_pos_file", str),
    ("density_z", "density_z_file", str),
    ("density_wt", "density_wt_file", str),
    ("density_jk", "density_jk_file", str),
    ("density_e", "density_e_file", str),
    ("Srandom_pos", "shape_rand_pos_file", str),
    ("Srandom_z", "shape_rand_z_file", str),
    ("Srandoms_wt", "shape_rand_wt_file", str),
    ("Srand_jk", "shape_rand_jk_file", str),
    ("Srand_patch", "shape_rand_patch_file", str),
    ("Drandom_pos", "density_rand_pos_file", str),
    ("Drandom_z", "density_rand_z_file", str),
    ("Drandoms_wt", "density_rand_wt_file", str),
    ("drand_jk", "density_rand_jk_file", str),
    ("distances", "distance_file", str),
    ("patch_file", "patches_file", str),
    ("out_file", "out_file", str),
    ("n_threads", "n_threads", int),
    ("n_shape", "n_shape", int),
    ("n_density", "n_density", int),
    ("n_Srand", "n_shape_rand", int),
    ("n_Drand", "n_density_rand", int),
    ("rand_subsample", "rand_subsample", int),
    ("n_jk", "n_jk_regions", int),
    ("n_patch", "n_patch", int),
    ("binR_min", "bin_r_min", float),
    ("binR_max", "bin_r_max", float),
    ("n_bins", "n_bins", int),
    ("lin_bin", "lin_bin", int),
    ("n_p_bin", "n_p_bin", int),
    ("pmin", "p_min", float),
    ("pmax", "p_max", float),
    ("z_min", "z_min", float),
    ("z_max", "z_max", float),
    ("dz", "dz", float),
    ("z_sep_min", "z_sep_min", float),
    ("z_sep_max", "z_sep_max", float),
    ("periodic_box", "periodic_box", int),
    ("box_size", "periodic_box_size", float),
]


@dataclass
class InpParams:
    """The positional .inp parameter set (data_info fields, data_def.h:46-96)."""

    which_corr: int = 0
    coordinates: int = 6
    estimator: int = 0
    data_sorted: int = 1
    use_comoving: int = 1
    do_jk: int = 1
    sig_crit: int = 0
    shape_pos_file: str = "0"
    shape_z_file: str = "0"
    shape_e_file: str = "0"
    shape_wt_file: str = "0"
    shape_jk_file: str = "0"
    shape_patch_file: str = "0"
    density_pos_file: str = "0"
    density_z_file: str = "0"
    density_wt_file: str = "0"
    density_jk_file: str = "0"
    density_e_file: str = "0"
    shape_rand_pos_file: str = "0"
    shape_rand_z_file: str = "0"
    shape_rand_wt_file: str = "0"
    shape_rand_jk_file: str = "0"
    shape_rand_patch_file: str = "0"
    density_rand_pos_file: str = "0"
    density_rand_z_file: str = "0"
    density_rand_wt_file: str = "0"
    density_rand_jk_file: str = "0"
    distance_file: str = "0"
    patches_file: str = "0"
    out_file: str = "out_"
    n_threads: int = 0
    n_shape: int = 0
    n_density: int = 0
    n_shape_rand: int = 0
    n_density_rand: int = 0
    rand_subsample: int = 0
    n_jk_regions: int = 0
    n_patch: int = 0
    bin_r_min: float = 0.1
    bin_r_max: float = 20.0
    n_bins: int = 10
    lin_bin: int = 0
    n_p_bin: int = 20
    p_min: float = -100.0
    p_max: float = 100.0
    z_min: float = 0.0
    z_max: float = 250.0
    dz: float = 0.0001
    z_sep_min: float = -100.0
    z_sep_max: float = 100.0
    periodic_box: int = 1
    periodic_box_size: float = 250.0

    def to_inp_text(self) -> str:
        lines = []
        for key, attr, kind in INP_KEYS:
            v = getattr(self, attr)
            if kind is float:
                lines.append(f"{key:<16s}{float(v)!r}")
            else:
                lines.append(f"{key:<16s}{v}")
        return "\n".join(lines) + "\n"

    def write(self, path: str) -> None:
        with open(path, "w") as f:
            f.write(self.to_inp_text())

    @classmethod
    def read(cls, path: str) -> "InpParams":
        """Positional reader: like data_ini, keys are ignored and order is the
        contract (initialization.cpp:70-130)."""
        toks = open(path).read().split()
        p = cls()
        it = iter(toks)
        for _key, attr, kind in INP_KEYS:
            next(it)  # key (ignored)
            v = next(it)
            if kind is int:
                setattr(p, attr, int(float(v)) if v.strip() not in ("",) else 0)
            elif kind is float:
                setattr(p, attr, float(v))
            else:
                setattr(p, attr, v)
        return p


# ---------------------------------------------------------------------------
# catalogues
# ---------------------------------------------------------------------------


@dataclass
class Catalog:
    """One catalogue in memory (SoA float64, as the reference reads it)."""

    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    w: np.ndarray | None = None
    e1: np.ndarray | None = None   # e1, or kappa (which_corr 3, 4) with e2 None
    e2: np.ndarray | None = None
    jk: np.ndarray | None = None
    e3: np.ndarray | None = None   # third orientation component (which_corr 5)

    @property
    def n(self) -> int:
        return int(self.x.shape[0])

    def sorted_by_z(self) -> "Catalog":
        o = np.argsort(self.z, kind="stable")
        return self.subset(o)

    def subset(self, idx) -> "Catalog":
        take = lambda a: None if a is None else np.ascontiguousarray(a[idx])
        return Catalog(take(self.x), take(self.y), take(self.z), take(self.w),
                       take(self.e1), take(self.e2), take(self.jk), take(self.e3))


def _wrap(v: np.ndarray, L: float) -> np.ndarray:
    v = np.mod(v, L)
    v[v >= L] = 0.0  # np.mod can return L for tiny negative inputs
    return v


def _to_f32_in_box(v: np.ndarray, L: float) -> np.ndarray:
    """Cast to float32 (the workload's stated position precision) and keep every
    value strictly inside [0, L): a float32 rounding up to L wraps to 0."""
    f = v.astype(np.float32)
    f[f >= np.float32(L)] = np.float32(0.0)
    return f.astype(np.float64)


def shapes(rng: np.random.Generator, n: int, sigma: float = 0.5):
    """e1, e2 ~ N(0, sigma^2) per component, resampled until |e| < 1."""
    e1 = rng.normal(0.0, sigma, n)
    e2 = rng.normal(0.0, sigma, n)
    bad = e1 * e1 + e2 * e2 >= 1.0
    while bad.any():
        k = int(bad.sum())
        e1[bad] = rng.normal(0.0, sigma, k)
        e2[bad] = rng.normal(0.0, sigma, k)
        bad = e1 * e1 + e2 * e2 >= 1.0
    return e1, e2


def jk_cubes(x, y, z, L: float, nside: int) -> np.ndarray:
    """Cubic jackknife sub-volumes: label = (ix*nside + iy)*nside + iz."""
    f = nside / L
    ix = np.minimum((x * f).astype(np.int64), nside - 1)
    iy = np.minimum((y * f).astype(np.int64), nside - 1)
    iz = np.minimum((z * f).astype(np.int64), nside - 1)
    return ((ix * nside + iy) * nside + iz).astype(np.int32)


def uniform_box(n: int, L: float, seed: int, *, nside_jk: int = 0,
                with_shapes: bool = False, float32: bool = False) -> Catalog:
    rng = np.random.default_rng(seed)
    xyz = rng.uniform(0.0, L, size=(3, n))
    if float32:
        xyz = np.stack([_to_f32_in_box(v, L) for v in xyz])
    x, y, z = (np.ascontiguousarray(v) for v in xyz)
    e1 = e2 = None
    if with_shapes:
        e1, e2 = shapes(rng, n)
    jk = jk_cubes(x, y, z, L, nside_jk) if nside_jk else None
    return Catalog(x, y, z, None, e1, e2, jk).sorted_by_z()


def with_kappa(cat: Catalog, seed: int) -> Catalog:
    """A copy carrying a per-galaxy scalar (kappa, or a mean-subtracted log mass as
    in the size notebook) in e1, e2 absent: one column in the e file."""
    rng = np.random.default_rng(seed)
    k = np.log10(rng.lognormal(0.0, 1.0, cat.n))
    k -= k.mean()
    return Catalog(cat.x, cat.y, cat.z, cat.w, k, None, cat.jk)


def with_orientation(cat: Catalog, seed: int) -> Catalog:
    """A copy carrying an un-normalised 3-D orientation (e1, e2, e3) -- the ED
    notebook's dark-matter axis -- with random lengths and a few zero vectors."""
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(3, cat.n)) * rng.uniform(0.2, 3.0, cat.n)
    v[:, :: max(1, cat.n // 7)] = 0.0
    return Catalog(cat.x, cat.y, cat.z, cat.w, v[0].copy(), v[1].copy(), cat.jk, v[2].copy())


def neyman_scott(n_parents: int, mean_children: float, sigma: float, L: float,
                 seed: int, *, nside_jk: int = 0, with_shapes: bool = True,
                 float32: bool = True) -> Catalog:
    """Poisson parents uniform in [0,L)^3, Poisson(mean) children each with an
    isotropic Gaussian offset, wrapped periodically."""
    rng = np.random.default_rng(seed)
    parents = rng.uniform(0.0, L, size=(n_parents, 3))
    counts = rng.poisson(mean_children, n_parents)
    n = int(counts.sum())
    pos = np.repeat(parents, counts, axis=0) + rng.normal(0.0, sigma, size=(n, 3))
    cols = []
    for d in range(3):
        v = _wrap(pos[:, d].copy(), L)
        cols.append(_to_f32_in_box(v, L) if float32 else v)
    x, y, z = (np.ascontiguousarray(c) for c in cols)
    e1 = e2 = None
    if with_shapes:
        e1, e2 = shapes(rng, n)
    jk = jk_cubes(x, y, z, L, nside_jk) if nside_jk else None
    return Catalog(x, y, z, None, e1, e2, jk).sorted_by_z()


# ---------------------------------------------------------------------------
# named workloads
# ---------------------------------------------------------------------------


@dataclass
class Workload:
    name: str
    params: InpParams
    shape: Catalog  # S sample
    density: Catalog  # D sample (same points for these cross-as-auto runs)
    extra: dict = field(default_factory=dict)


def _box_params(*, which_corr, L, rmin, rmax, nrp, npi, pmax, njk, n) -> InpParams:
    return InpParams(which_corr=which_corr, coordinates=6, estimator=0,
                     data_sorted=1, use_comoving=1, do_jk=1 if njk else 0,
                     sig_crit=0, n_shape=n, n_density=n, n_jk_regions=njk,
                     bin_r_min=rmin, bin_r_max=rmax, n_bins=nrp, lin_bin=0,
                     n_p_bin=npi, p_min=-pmax, p_max=pmax, z_min=0.0, z_max=L,
                     dz=0.0001, z_sep_min=-pmax, z_sep_max=pmax, periodic_box=1,
                     periodic_box_size=L)


def box_uniform_wgg(n: int = 20000, seed: int = 0) -> Workload:
    L = 250.0
    cat = uniform_box(n, L, seed, nside_jk=2)
    p = _box_params(which_corr=0, L=L, rmin=0.1, rmax=20.0, nrp=10, npi=20,
                    pmax=100.0, njk=8, n=cat.n)
    return Workload("box_uniform_wgg_20k", p, cat, cat)


def box_ns_wgp(seed: int = 0, n_parents: int = 2000) -> Workload:
    L = 500.0
    cat = neyman_scott(n_parents, 100.0, 2.0, L, seed, nside_jk=4)
    p = _box_params(which_corr=1, L=L, rmin=0.1, rmax=60.0, nrp=20, npi=40,
                    pmax=100.0, njk=64, n=cat.n)
    return Workload("box_ns_wgp_200k", p, cat, cat)


def box_ns_ed_rmu(seed: int = 0, n_parents: int = 2000) -> Workload:
    """The 200k clustered box with 3-D orientations: ED (which_corr 5) in r-mu
    (coordinates 7), 20 log r bins 0.1-60, 10 mu bins, 64 jackknife cubes."""
    L = 500.0
    cat = with_orientation(neyman_scott(n_parents, 100.0, 2.0, L, seed, nside_jk=4), seed + 1)
    p = _box_params(which_corr=5, L=L, rmin=0.1, rmax=60.0, nrp=20, npi=10, pmax=1.0,
                    njk=64, n=cat.n)
    p.coordinates = 7
    return Workload("box_ns_ed_rmu_200k", p, cat, cat)


def box_ns_kappa(seed: int = 0, n_parents: int = 2000) -> Workload:
    """The 200k clustered box with a per-galaxy scalar: kappa-density
    (which_corr 3), the headline binning."""
    L = 500.0
    cat = with_kappa(neyman_scott(n_parents, 100.0, 2.0, L, seed, nside_jk=4), seed + 1)
    p = _box_params(which_corr=3, L=L, rmin=0.1, rmax=60.0, nrp=20, npi=40, pmax=100.0,
                    njk=64, n=cat.n)
    return Workload("box_ns_kappa_200k", p, cat, cat)


def box_ns_large_wpp(seed: int = 0, n_parents: int = 200000) -> Workload:
    L = 1000.0
    cat = neyman_scott(n_parents, 100.0, 3.0, L, seed, nside_jk=5)
    p = _box_params(which_corr=2, L=L, rmin=0.1, rmax=100.0, nrp=25, npi=50,
                    pmax=100.0, njk=125, n=cat.n)
    return Workload("box_ns_wpp_20M", p, cat, cat)


def box_batch_sizes(n_boxes: int = 64, seed: int = 0, lo: float = 1e4,
                    hi: float = 4e5) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n_boxes)).astype(np.int64)


def box_batch_wpp(n_boxes: int = 64, seed: int = 0, scale: float = 1.0) -> list:
    """64 uneven uniform sub-boxes (L=200), each a w++ job with 27 cubes.  The
    bin ranges (0.1-60 in r_p, +-100 in Pi) follow the 200k clustered box."""
    L = 200.0
    sizes = box_batch_sizes(n_boxes, seed)
    out = []
    for b, nb in enumerate(sizes):
        nb = max(2, int(nb * scale))
        cat = uniform_box(nb, L, seed * 1000 + b + 1, nside_jk=3, with_shapes=True)
        p = _box_params(which_corr=2, L=L, rmin=0.1, rmax=60.0, nrp=20, npi=40,
                        pmax=100.0, njk=27, n=cat.n)
        out.append(Workload(f"box_batch_{b}", p, cat, cat))
    return out


# ---------------------------------------------------------------------------
# writers (Gen_inp_Periodic_box.ipynb write_data / inp_gen formats)
# ---------------------------------------------------------------------------


def write_catalog(prefix: str, cat: Catalog, *, write_e: bool = True,
                  write_w: bool = True) -> dict:
    """Write ``<prefix>_pos.dat`` etc. and return the file names ("0" where a
    file is not written, which the reference reads as "absent")."""
    names = {"pos": prefix + "_pos.dat", "z": prefix + "_z.dat", "e": "0",
             "wt": "0", "jk": "0"}
    np.savetxt(names["pos"], np.column_stack((cat.x, cat.y)))
    np.savetxt(names["z"], cat.z)
    if cat.jk is not None:
        names["jk"] = prefix + "_jk.dat"
        np.savetxt(names["jk"], cat.jk, fmt="%i")
    if write_e and cat.e1 is not None:
        # one column (kappa), two (e1, e2) or three (the ED orientation)
        names["e"] = prefix + "_e.dat"
        cols = [c for c in (cat.e1, cat.e2, cat.e3) if c is not None]
        np.savetxt(names["e"], np.column_stack(cols))
    if write_w and cat.w is not None:
        names["wt"] = prefix + "_wt.dat"
        np.savetxt(names["wt"], cat.w)
    return names


def write_box_run(dirpath: str, wl: Workload, *, same_files: bool = True,
                  n_threads: int = 0) -> str:
    """Write the S and D catalogues and the .inp for a periodic-box cross run;
    returns the .inp path.  With ``same_files`` the density sample points to the
    shape sample's files (file_nameD = file_nameS in the notebooks)."""
    os.makedirs(dirpath, exist_ok=True)
    os.makedirs(os.path.join(dirpath, "out"), exist_ok=True)
    p = wl.params
    s = write_catalog(os.path.join(dirpath, "S"), wl.shape)
    d = s if same_files else write_catalog(os.path.join(dirpath, "D"), wl.density)
    p.shape_pos_file, p.shape_z_file, p.shape_e_file = s["pos"], s["z"], s["e"]
    p.shape_wt_file, p.shape_jk_file = s["wt"], s["jk"]
    p.density_pos_file, p.density_z_file = d["pos"], d["z"]
    p.density_wt_file, p.density_jk_file, p.density_e_file = d["wt"], d["jk"], d["e"]
    p.out_file = os.path.join(dirpath, "out", "run_")
    p.n_threads = n_threads
    p.n_shape, p.n_density = wl.shape.n, wl.density.n
    inp = os.path.join(dirpath, "run.inp")
    p.write(inp)
    return inp


# ---------------------------------------------------------------------------
# sky catalogues (coordinates 0: RA, Dec in degrees, redshift)
# ---------------------------------------------------------------------------

C_KMS = 299792.458


@dataclass
class DistanceTable:
    """Rows of the distances file read by da_Z (initialization.cpp:23-60):
    z, H(z) [km/s per Mpc/h], D_A, D_C, and a fifth column that da_Z stores as
    the transverse distance when use_comoving is 1 (Gen_inp_HSC writes the
    comoving distance there; so does this generator)."""

    z: np.ndarray
    H: np.ndarray
    DA: np.ndarray
    DC: np.ndarray

    @property
    def transverse(self) -> np.ndarray:
        return self.DC

    def write(self, path: str) -> None:
        np.savetxt(path, np.column_stack((self.z, self.H, self.DA, self.DC, self.DC)),
                   fmt="%.18e")


def flat_lcdm_table(z_max: float, dz: float, omega_m: float = 0.3,
                    h0: float = 100.0) -> DistanceTable:
    """Flat LCDM distances on the grid z_k = k dz, k = 0 .. ceil((z_max+1)/dz)+20
    (the length data_ini allocates), D_C by the trapezoid rule."""
    n = int(np.ceil((z_max + 1.0) / dz)) + 21
    z = np.arange(n, dtype=np.float64) * dz
    H = h0 * np.sqrt(omega_m * (1.0 + z) ** 3 + 1.0 - omega_m)
    inv = C_KMS / H
    dc = np.concatenate(([0.0], np.cumsum(0.5 * (inv[1:] + inv[:-1]) * dz)))
    return DistanceTable(z, H, dc / (1.0 + z), dc)


def jk_sky_grid(ra, dec, ra_range, dec_range, n_ra: int, n_dec: int) -> np.ndarray:
    """Jackknife regions on an RA/Dec grid: label = i_ra * n_dec + i_dec."""
    fa = n_ra / (ra_range[1] - ra_range[0])
    fd = n_dec / (dec_range[1] - dec_range[0])
    ia = np.clip(((ra - ra_range[0]) * fa).astype(np.int64), 0, n_ra - 1)
    idd = np.clip(((dec - dec_range[0]) * fd).astype(np.int64), 0, n_dec - 1)
    return (ia * n_dec + idd).astype(np.int32)


def sky_patch(n: int, seed: int, table: DistanceTable, *, ra_deg: float = 10.0,
              dec_deg: float = 10.0, chi_range=(500.0, 1500.0), nside_jk: int = 10,
              with_shapes: bool = False, weights: bool = False) -> Catalog:
    """Points uniform on the patch RA in [0, ra_deg), sin(Dec) uniform on
    [0, sin(dec_deg)), comoving distance with p(chi) ~ chi^2 on chi_range,
    converted to redshift through the table; sorted by redshift."""
    rng = np.random.default_rng(seed)
    ra = rng.uniform(0.0, ra_deg, n)
    dec = np.degrees(np.arcsin(rng.uniform(0.0, np.sin(np.radians(dec_deg)), n)))
    c0, c1 = chi_range
    chi = np.cbrt(rng.uniform(c0 ** 3, c1 ** 3, n))
    z = np.interp(chi, table.DC, table.z)
    e1 = e2 = None
    if with_shapes:
        e1, e2 = shapes(rng, n)
    w = rng.uniform(0.5, 1.5, n) if weights else None
    jk = jk_sky_grid(ra, dec, (0.0, ra_deg), (0.0, dec_deg), nside_jk, nside_jk) \
        if nside_jk else None
    return Catalog(ra, dec, z, w, e1, e2, jk).sorted_by_z()


@dataclass
class SkyWorkload:
    name: str
    params: InpParams
    table: DistanceTable
    shape: Catalog       # S
    density: Catalog     # D
    shape_rand: Catalog  # Rs
    density_rand: Catalog  # Rd


def _sky_params(*, which_corr, rmin, rmax, nrp, npi, pmax, njk, z_max=1.0) -> InpParams:
    return InpParams(which_corr=which_corr, coordinates=0, estimator=0, data_sorted=1,
                     use_comoving=1, do_jk=1 if njk else 0, sig_crit=0,
                     n_jk_regions=njk, bin_r_min=rmin, bin_r_max=rmax, n_bins=nrp,
                     lin_bin=0, n_p_bin=npi, p_min=-pmax, p_max=pmax, z_min=0.0,
                     z_max=z_max, dz=0.0001, z_sep_min=0.0, z_sep_max=0.0,
                     periodic_box=0, periodic_box_size=0.0)


def sky_wgp(n_data: int = 500000, n_rand: int = 5000000, seed: int = 0,
            which_corr: int = 1) -> SkyWorkload:
    """Sky survey: data (with shapes and U(0.5,1.5) weights) and randoms on a
    10x10 degree patch, chi 500-1500 Mpc/h, 15 log r_p bins 0.3-60, 30 Pi bins
    over +-60, 100 jackknife regions on a 10x10 RA/Dec grid; terms SRd, RsRd, SD,
    DRs.  S and D are the same points, Rs and Rd the same randoms."""
    p = _sky_params(which_corr=which_corr, rmin=0.3, rmax=60.0, nrp=15, npi=30, pmax=60.0,
                    njk=100)
    t = flat_lcdm_table(p.z_max, p.dz)
    d = sky_patch(n_data, seed, t, with_shapes=True, weights=True)
    r = sky_patch(n_rand, seed + 1, t)
    return SkyWorkload(f"sky_wgp_{n_data}_{n_rand}", p, t, d, d, r, r)


def write_sky_run(dirpath: str, wl: SkyWorkload, *, n_threads: int = 0,
                  same_files: bool = True) -> str:
    """Write the four catalogues, the distances file and the .inp of a sky cross
    run (terms SRd, RsRd, SD, DRs); returns the .inp path."""
    os.makedirs(os.path.join(dirpath, "out"), exist_ok=True)
    p = wl.params
    s = write_catalog(os.path.join(dirpath, "S"), wl.shape)
    d = s if same_files else write_catalog(os.path.join(dirpath, "D"), wl.density)
    rs = write_catalog(os.path.join(dirpath, "Rs"), wl.shape_rand, write_e=False)
    rd = rs if same_files else write_catalog(os.path.join(dirpath, "Rd"), wl.density_rand,
                                             write_e=False)
    dist = os.path.join(dirpath, "distances.dat")
    wl.table.write(dist)
    p.shape_pos_file, p.shape_z_file, p.shape_e_file = s["pos"], s["z"], s["e"]
    p.shape_wt_file, p.shape_jk_file = s["wt"], s["jk"]
    p.density_pos_file, p.density_z_file = d["pos"], d["z"]
    p.density_wt_file, p.density_jk_file, p.density_e_file = d["wt"], d["jk"], d["e"]
    p.shape_rand_pos_file, p.shape_rand_z_file = rs["pos"], rs["z"]
    p.shape_rand_wt_file, p.shape_rand_jk_file = rs["wt"], rs["jk"]
    p.density_rand_pos_file, p.density_rand_z_file = rd["pos"], rd["z"]
    p.density_rand_wt_file, p.density_rand_jk_file = rd["wt"], rd["jk"]
    p.distance_file = dist
    p.out_file = os.path.join(dirpath, "out", "run_")
    p.n_threads = n_threads
    p.n_shape, p.n_density = wl.shape.n, wl.density.n
    p.n_shape_rand, p.n_density_rand = wl.shape_rand.n, wl.density_rand.n
    inp = os.path.join(dirpath, "run.inp")
    p.write(inp)
    return inp


def derived_z_sep(p: InpParams, table: DistanceTable) -> tuple:
    """z_sep_max / z_sep_min as data_ini derives them for coordinates 0
    (initialization.cpp:223-276): p_max * H(z_idx) / 300000 + 0.001 with
    z_idx = ceil(z_max / dz)."""
    k = int(np.ceil(p.z_max / p.dz))
    return (p.p_max * table.H[k] / 300000.0 + 0.001,
            p.p_min * table.H[k] / 300000.0 - 0.001)
