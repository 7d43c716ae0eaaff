"""Crystal data (the cr_* arrays of discus/prog/crystal_mod.f90:25-138) and
seeded synthetic structures for the benchmark workloads.

A crystal is stored in "DISCUS order" (celltoindex, discus/prog/celltoindex.f90:7-25):
atom index = ((k*icc1*icc2 + j*icc1 + i) * ncatoms + site), cell x fastest,
so that four_aver can fold atoms per unit cell.  Vacancies keep their slot and
get type 0 (VOID), as DISCUS does; type loops start at 1 and skip them
(fourier_sup.f90:224).

All generators use numpy's PCG64 with an explicit seed.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi


def reciprocal_metric(a, b, c, alpha, beta, gamma):
    """cr_rten from lattice constants, as `lattice` computes it
    (discus/prog/spcgr_apply.f90:3538-3658): reciprocal constants a*, alpha*
    from the direct ones, then the metric tensor of (a*, alpha*)."""
    ca, cb, cg = (math.cos(math.radians(x)) for x in (alpha, beta, gamma))
    sa, sb, sg = (math.sin(math.radians(x)) for x in (alpha, beta, gamma))
    vol = math.sqrt(1 - ca * ca - cb * cb - cg * cg + 2 * ca * cb * cg) * a * b * c
    ar = [b * c * sa / vol, c * a * sb / vol, a * b * sg / vol]
    cos_r = [(cb * cg - ca) / (sb * sg), (cg * ca - cb) / (sg * sa), (ca * cb - cg) / (sa * sb)]
    g = np.empty((3, 3))
    for i in range(3):
        for j in range(3):
            if i == j:
                g[i, j] = ar[i] * ar[i]
            else:
                k = 3 - i - j
                g[i, j] = ar[i] * ar[j] * cos_r[k]
    return g


def direct_metric(a, b, c, alpha, beta, gamma):
    """cr_gten from lattice constants (spcgr_apply.f90:3538-3658): a_i a_j cos."""
    a0 = (a, b, c)
    cw = [math.cos(math.radians(x)) for x in (alpha, beta, gamma)]
    g = np.empty((3, 3))
    for i in range(3):
        for j in range(3):
            g[i, j] = a0[i] * a0[i] if i == j else a0[i] * a0[j] * cw[3 - i - j]
    return g


@dataclass
class PowderSpec:
    """The powder menu state powder_complete reads (powder_mod.f90): steps and
    shift along h, k, l, the d* sphere, the Q scale and the preferred
    orientation.  a0/gten are the crystal's cr_a0/cr_gten."""
    a0: tuple
    gten: np.ndarray
    hkl_del: tuple = (0.05, 0.05, 0.05)
    hkl_shift: tuple = (0.0, 0.0, 0.0)
    ds_max: float = 0.8
    qmin: float = 0.5
    qmax: float = 5.0
    deltaq: float = 0.001
    l_all: bool = True
    pref_type: int = 0
    pref_hkl: tuple = (0.0, 0.0, 1.0)
    pref_g1: float = 0.0
    pref_g2: float = 0.0
    slabs: int = 0                       # device h-slabs, 0 = automatic (no DISCUS counterpart)

    @classmethod
    def for_lattice(cls, a, b, c, alpha=90.0, beta=90.0, gamma=90.0, **kw):
        return cls(a0=(a, b, c), gten=direct_metric(a, b, c, alpha, beta, gamma), **kw)

    def to_c(self):
        p = _abi.Powder()
        for k in range(3):
            p.hkl_del[k] = float(self.hkl_del[k])
            p.hkl_shift[k] = float(self.hkl_shift[k])
            p.a0[k] = float(self.a0[k])
            p.pref_hkl[k] = float(self.pref_hkl[k])
        for k, v in enumerate(np.asarray(self.gten, dtype=np.float64).reshape(-1, order="F")):
            p.gten[k] = float(v)
        p.ds_max, p.qmin, p.qmax, p.deltaq = float(self.ds_max), float(self.qmin), float(self.qmax), float(self.deltaq)
        p.l_all = 1 if self.l_all else 0
        p.pref_type = int(self.pref_type)
        p.pref_g1, p.pref_g2 = float(self.pref_g1), float(self.pref_g2)
        p.slabs = int(self.slabs)
        return p

    @property
    def n_pkt(self):
        """powder.f90:1957: NINT((qmax + deltaq - qmin) / deltaq) + 2."""
        x = (self.qmax + self.deltaq - self.qmin) / self.deltaq
        return int(math.floor(x + 0.5)) + 2

    def q(self):
        """Q of pow_qsp(0:n_pkt)."""
        return self.qmin + self.deltaq * np.arange(self.n_pkt + 1)


@dataclass
class CrystalData:
    pos: np.ndarray            # (natoms, 3) float64, lattice units
    iscat: np.ndarray          # (natoms,) int32, 0 = VOID
    nscat: int
    ncatoms: int
    icc: tuple
    rten: np.ndarray           # (3, 3)
    scat: np.ndarray           # (nscat+1, 11): c, a1, b1, ..., a5, b5
    occ: np.ndarray            # (nscat+1,)
    dw: np.ndarray             # (nscat+1,)
    dim0: tuple = (0.0, 0.0, 0.0)
    delfr: np.ndarray | None = None
    delfi: np.ndarray | None = None
    atom_occ: np.ndarray | None = None   # (natoms,) float32, not part of DISCUS
    name: str = ""
    # anisotropic ADPs (crystal_mod cr_is_anis, cr_iscat(3,:), cr_anis_full, cr_ar)
    ianis: np.ndarray | None = None      # (natoms,) int32, ADP type 1..nanis
    anis_full: np.ndarray | None = None  # (nanis, 6) U11 U22 U33 U23 U13 U12, A^2
    ar: tuple = (0.0, 0.0, 0.0)          # reciprocal cell lengths, 1/A
    dim_lo: tuple | None = None          # cr_dim(:,1); None = min over the positions
    isym: np.ndarray | None = None       # (natoms,) int32, cr_iscat(2,:): generating symmetry (DISCAMB)
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        self.pos = np.ascontiguousarray(self.pos, dtype=np.float64)
        self.iscat = np.ascontiguousarray(self.iscat, dtype=np.int32)
        self.rten = np.asarray(self.rten, dtype=np.float64)
        self.scat = np.ascontiguousarray(self.scat, dtype=np.float64)
        self.occ = np.ascontiguousarray(self.occ, dtype=np.float64)
        self.dw = np.ascontiguousarray(self.dw, dtype=np.float64)
        if self.delfr is None:
            self.delfr = np.zeros(self.nscat + 1)
        if self.delfi is None:
            self.delfi = np.zeros(self.nscat + 1)
        if self.atom_occ is not None:
            self.atom_occ = np.ascontiguousarray(self.atom_occ, dtype=np.float32)
        if self.ianis is not None:
            self.ianis = np.ascontiguousarray(self.ianis, dtype=np.int32)
            self.anis_full = np.ascontiguousarray(np.asarray(self.anis_full, dtype=np.float64).reshape(-1, 6))
        if self.dim_lo is None:
            self.dim_lo = tuple(float(x) for x in self.pos.min(axis=0)) if len(self.pos) else (0.0, 0.0, 0.0)
        if self.isym is not None:
            self.isym = np.ascontiguousarray(self.isym, dtype=np.int32)

    @property
    def is_anis(self):
        return self.ianis is not None

    @property
    def natoms(self):
        return int(self.pos.shape[0])

    def n_scattering(self):
        return int(np.count_nonzero((self.iscat >= 1) & (self.iscat <= self.nscat)))

    def to_c(self, pos_ptr=None, iscat_ptr=None, occ_ptr=None, ianis_ptr=None):
        """Fill a dgpu_crystal; pointer overrides allow device arrays."""
        cr = _abi.Crystal()
        cr.natoms = self.natoms
        cr.pos = pos_ptr if pos_ptr is not None else _abi.dptr(self.pos)
        cr.iscat = iscat_ptr if iscat_ptr is not None else _abi.iptr(self.iscat)
        if occ_ptr is not None:
            cr.atom_occ = occ_ptr
        else:
            cr.atom_occ = _abi.fptr(self.atom_occ)
        cr.nscat = self.nscat
        cr.ncatoms = self.ncatoms
        for k in range(3):
            cr.icc[k] = int(self.icc[k])
            cr.dim0[k] = float(self.dim0[k])
        rt = np.asfortranarray(self.rten).reshape(-1, order="F")
        for k in range(9):
            cr.rten[k] = float(rt[k])
        cr.scat = _abi.dptr(self.scat)
        cr.occ = _abi.dptr(self.occ)
        cr.dw = _abi.dptr(self.dw)
        cr.delfr = _abi.dptr(self.delfr)
        cr.delfi = _abi.dptr(self.delfi)
        for k in range(3):
            cr.ar[k] = float(self.ar[k])
            cr.dim_lo[k] = float(self.dim_lo[k])
        if self.ianis is not None:
            cr.is_anis = 1
            cr.nanis = int(self.anis_full.shape[0])
            cr.ianis = ianis_ptr if ianis_ptr is not None else _abi.iptr(self.ianis)
            cr.anis_full = _abi.dptr(self.anis_full)
        if self.isym is not None:
            cr.isym = _abi.iptr(self.isym)
        return cr

    def with_positions(self, pos, atom_occ=None):
        return CrystalData(pos=pos, iscat=self.iscat, nscat=self.nscat, ncatoms=self.ncatoms,
                           icc=self.icc, rten=self.rten, scat=self.scat, occ=self.occ,
                           dw=self.dw, dim0=self.dim0, delfr=self.delfr, delfi=self.delfi,
                           atom_occ=self.atom_occ if atom_occ is None else atom_occ,
                           name=self.name, ianis=self.ianis, anis_full=self.anis_full, ar=self.ar,
                           dim_lo=self.dim_lo, isym=self.isym)


@dataclass
class GridData:
    eck: np.ndarray   # (3, 4) corners ll, lr, ul, tl
    vi: np.ndarray    # (3, 3) increment vectors (columns)
    inc: tuple

    def __post_init__(self):
        self.eck = np.asarray(self.eck, dtype=np.float64).reshape(3, 4)
        self.vi = np.asarray(self.vi, dtype=np.float64).reshape(3, 3)
        self.inc = tuple(int(x) for x in self.inc)

    @classmethod
    def from_corners(cls, ll, lr, ul, tl=None, inc=(121, 121, 1)):
        """vi from corners and point counts, as the fourier menu does with
        ll/lr/ul/tl and nabs/nord/ntop."""
        ll, lr, ul = (np.asarray(x, dtype=np.float64) for x in (ll, lr, ul))
        tl = ll.copy() if tl is None else np.asarray(tl, dtype=np.float64)
        vi = np.zeros((3, 3))
        if inc[0] > 1:
            vi[:, 0] = (lr - ll) / (inc[0] - 1)
        if inc[1] > 1:
            vi[:, 1] = (ul - ll) / (inc[1] - 1)
        if inc[2] > 1:
            vi[:, 2] = (tl - ll) / (inc[2] - 1)
        eck = np.stack([ll, lr, ul, tl], axis=1)
        return cls(eck=eck, vi=vi, inc=inc)

    @property
    def npoints(self):
        return int(np.prod(self.inc))

    def to_c(self):
        g = _abi.Grid()
        e = self.eck.reshape(-1, order="F")
        v = self.vi.reshape(-1, order="F")
        for k in range(12):
            g.eck[k] = float(e[k])
        for k in range(9):
            g.vi[k] = float(v[k])
        for k in range(3):
            g.inc[k] = self.inc[k]
        return g

    def hkl(self):
        """(3, n1, n2, n3) array of the grid's h vectors."""
        n1, n2, n3 = self.inc
        i = np.arange(n1)[:, None, None]
        j = np.arange(n2)[None, :, None]
        k = np.arange(n3)[None, None, :]
        return (self.eck[:, 0, None, None, None] + self.vi[:, 0, None, None, None] * i
                + self.vi[:, 1, None, None, None] * j + self.vi[:, 2, None, None, None] * k)


def random_form_factors(rng, nscat, b_iso=0.5, power=4):
    """Seeded 4-Gaussian + constant X-ray form factors:
    a_i ~ U(0.5,10), b_i ~ U(0.5,50), c ~ U(0,2); cr_scat order c,a1,b1,...
    (fourier.f90:751-774)."""
    scat = np.zeros((nscat + 1, 11))
    for t in range(1, nscat + 1):
        scat[t, 0] = rng.uniform(0.0, 2.0)
        for i in range(1, power + 1):
            scat[t, 2 * i - 1] = rng.uniform(0.5, 10.0)
            scat[t, 2 * i] = rng.uniform(0.5, 50.0)
    occ = np.ones(nscat + 1)
    dw = np.full(nscat + 1, b_iso)
    dw[0] = 0.0
    return scat, occ, dw


def _cells(icc):
    """Cell origins in DISCUS order (x fastest)."""
    i, j, k = np.meshgrid(np.arange(icc[0]), np.arange(icc[1]), np.arange(icc[2]), indexing="ij")
    return np.stack([i.ravel(order="F"), j.ravel(order="F"), k.ravel(order="F")], axis=1).astype(np.float64)


def build_periodic(sites, types, icc, a_lat, rng, sigma_ang=0.0, fp32=False):
    """Sites (ns,3) fractional, types (ns,), cells icc -> pos, iscat."""
    sites = np.asarray(sites, dtype=np.float64)
    cells = _cells(icc)
    pos = (cells[:, None, :] + sites[None, :, :]).reshape(-1, 3)
    iscat = np.tile(np.asarray(types, dtype=np.int32), cells.shape[0])
    if sigma_ang > 0:
        pos = pos + rng.normal(0.0, 1.0, size=pos.shape) * (sigma_ang / np.asarray(a_lat))
    if fp32:
        pos = pos.astype(np.float32).astype(np.float64)
    return pos, iscat


def perovskite_plane(seed=1, cells=10, vacancy=0.3, sigma=0.01, fp32=False):
    """Cubic perovskite-like crystal a = 4.0 A: A(0,0,0) B(1/2,1/2,1/2),
    O(1/2,1/2,0),(1/2,0,1/2),(0,1/2,1/2); 30% of B sites VOID; Gaussian
    displacements sigma per axis; isotropic B = 0.5 A^2; hk0 plane
    201 x 201 from (-5,-5,0) step 0.05."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = 4.0
    sites = [[0, 0, 0], [0.5, 0.5, 0.5], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]]
    types = [1, 2, 3, 3, 3]
    icc = (cells, cells, cells)
    pos, iscat = build_periodic(sites, types, icc, a, rng, sigma, fp32)
    bsite = iscat == 2
    vac = rng.random(iscat.shape[0]) < vacancy
    iscat = np.where(bsite & vac, 0, iscat).astype(np.int32)
    scat, occ, dw = random_form_factors(rng, 3, b_iso=0.5)
    cr = CrystalData(pos=pos, iscat=iscat, nscat=3, ncatoms=5, icc=icc,
                     rten=reciprocal_metric(a, a, a, 90, 90, 90), scat=scat, occ=occ, dw=dw,
                     name="perovskite-10x10x10")
    grid = GridData.from_corners((-5, -5, 0), (5, -5, 0), (-5, 5, 0), inc=(201, 201, 1))
    return cr, grid


def _ising_sro(rng, nsub, icc, sweeps, j_over_kt):
    """Composition-conserving Metropolis exchange on the fcc NN Ising model,
    E = -J sum_nn s_i s_j.  fcc = 4 simple-cubic sublattices; the 12 nearest
    neighbours of a site lie on the other 3, so all swaps between two sites of
    the same sublattice are independent and are done in one vectorised step."""
    n1, n2, n3 = icc
    tot = 4 * n1 * n2 * n3
    spin = np.where(rng.permutation(tot) < tot // 2, 1, -1).astype(np.int8).reshape(4, n1, n2, n3)
    # neighbour offsets: for sublattice s at cell c, NN on sublattice t at cell c + d
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    nbr = {s: [] for s in range(4)}
    for s in range(4):
        for t in range(4):
            if t == s:
                continue
            for dx in (-1, 0, 1):
                for dy in (-1, 0, 1):
                    for dz in (-1, 0, 1):
                        d = basis[t] + np.array([dx, dy, dz]) - basis[s]
                        if abs(np.dot(d, d) - 0.5) < 1e-9:
                            nbr[s].append((t, dx, dy, dz))
    for s in range(4):
        assert len(nbr[s]) == 12

    def field(s):
        f = np.zeros((n1, n2, n3), dtype=np.int32)
        for (t, dx, dy, dz) in nbr[s]:
            f += np.roll(spin[t], shift=(-dx, -dy, -dz), axis=(0, 1, 2))
        return f

    nsite = n1 * n2 * n3
    for _ in range(sweeps):
        for s in range(4):
            f = field(s).ravel()
            sp = spin[s].ravel().copy()
            perm = rng.permutation(nsite)
            a_idx = perm[: nsite // 2]
            b_idx = perm[nsite // 2: 2 * (nsite // 2)]
            diff = sp[a_idx] != sp[b_idx]
            # flip energy dE_i = 2 J s_i f_i (E = -J sum s s); a swap of unlike
            # spins flips both (same-sublattice sites are never neighbours)
            de = 2.0 * j_over_kt * (sp[a_idx] * f[a_idx] + sp[b_idx] * f[b_idx])
            acc = diff & (rng.random(a_idx.shape[0]) < np.exp(-np.maximum(de, 0.0)))
            ta = sp[a_idx[acc]].copy()
            sp[a_idx[acc]] = sp[b_idx[acc]]
            sp[b_idx[acc]] = ta
            spin[s] = sp.reshape(n1, n2, n3)
    return spin


def fcc_alloy_volume(seed=2, cells=50, sweeps=20, j_over_kt=0.1, sigma=0.02, inc=101, step=0.08):
    """fcc binary alloy a = 3.6 A, cells^3 x 4 atoms, 50/50 with SRO from
    NN Ising exchange sweeps, Gaussian displacements sigma, FP32-representable
    coordinates; 3D grid h,k,l in [-4,4] step 0.08 (101^3)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = 3.6
    icc = (cells, cells, cells)
    spin = _ising_sro(rng, 4, icc, sweeps, j_over_kt)
    sites = [[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]]
    pos, _ = build_periodic(sites, [1, 1, 1, 1], icc, a, rng, sigma, fp32=True)
    # DISCUS order: cell (x fastest) then site
    sp = np.stack([spin[s].ravel(order="F") for s in range(4)], axis=1).ravel()
    iscat = np.where(sp > 0, 1, 2).astype(np.int32)
    scat, occ, dw = random_form_factors(rng, 2, b_iso=0.5)
    cr = CrystalData(pos=pos, iscat=iscat, nscat=2, ncatoms=4, icc=icc,
                     rten=reciprocal_metric(a, a, a, 90, 90, 90), scat=scat, occ=occ, dw=dw,
                     name=f"fcc-alloy-{cells}^3")
    hmax = step * (inc - 1) / 2
    grid = GridData.from_corners((-hmax, -hmax, -hmax), (hmax, -hmax, -hmax), (-hmax, hmax, -hmax),
                                 (-hmax, -hmax, hmax), inc=(inc, inc, inc))
    return cr, grid


def hex_layers_plane(seed=3, na=200, nc=20, p_fault=0.1, vacancy=0.02, inc=1001, hmax=10.0):
    """Layered hexagonal crystal a = 2.46, c = 6.7 A, 2 atoms/cell
    ((0,0,0), (1/3,2/3,1/2)), na x na x nc cells; each layer shifted by
    (1/3,2/3,0) with probability p; 2% VOID; FP32 coordinates; h0l plane
    inc x inc over h,l in [-hmax,hmax]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    icc = (na, na, nc)
    sites = [[0, 0, 0], [1.0 / 3.0, 2.0 / 3.0, 0.5]]
    pos, iscat = build_periodic(sites, [1, 2], icc, (2.46, 2.46, 6.7), rng, 0.0, fp32=False)
    shifts = np.zeros((nc, 3))
    cur = np.zeros(3)
    for k in range(nc):
        if k > 0 and rng.random() < p_fault:
            cur = cur + np.array([1.0 / 3.0, 2.0 / 3.0, 0.0])
        shifts[k] = cur
    layer = np.floor(pos[:, 2]).astype(np.int64)
    pos = pos + shifts[np.clip(layer, 0, nc - 1)]
    pos = pos.astype(np.float32).astype(np.float64)
    vac = rng.random(iscat.shape[0]) < vacancy
    iscat = np.where(vac, 0, iscat).astype(np.int32)
    scat, occ, dw = random_form_factors(rng, 2, b_iso=0.5)
    cr = CrystalData(pos=pos, iscat=iscat, nscat=2, ncatoms=2, icc=icc,
                     rten=reciprocal_metric(2.46, 2.46, 6.7, 90, 90, 120), scat=scat, occ=occ,
                     dw=dw, name=f"hex-layers-{na}x{na}x{nc}")
    grid = GridData.from_corners((-hmax, 0, -hmax), (hmax, 0, -hmax), (-hmax, 0, hmax), inc=(inc, inc, 1))
    return cr, grid


def rocksalt_volume(seed=4, cells=(25, 25, 20), sigma=0.0, occ_pm=0.0, inc=65, step=0.1):
    """Rock salt a = 5.64 A, 8 atoms/cell (Na 4, Cl 4); optional Gaussian
    displacements and per-atom occupancies 1 + U(-occ_pm, occ_pm);
    3D grid h,k,l in [-3.2,3.2] step 0.1 (65^3)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = 5.64
    fcc = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    sites = np.concatenate([fcc, fcc + np.array([0.5, 0.0, 0.0])])
    sites = sites % 1.0
    pos, iscat = build_periodic(sites, [1, 1, 1, 1, 2, 2, 2, 2], cells, a, rng, sigma, fp32=True)
    scat, occ, dw = random_form_factors(rng, 2, b_iso=0.5)
    aocc = None
    if occ_pm > 0:
        aocc = (1.0 + rng.uniform(-occ_pm, occ_pm, size=iscat.shape[0])).astype(np.float32)
    cr = CrystalData(pos=pos, iscat=iscat, nscat=2, ncatoms=8, icc=cells,
                     rten=reciprocal_metric(a, a, a, 90, 90, 90), scat=scat, occ=occ, dw=dw,
                     atom_occ=aocc, name="rocksalt-25x25x20")
    hmax = step * (inc - 1) / 2
    grid = GridData.from_corners((-hmax, -hmax, -hmax), (hmax, -hmax, -hmax), (-hmax, hmax, -hmax),
                                 (-hmax, -hmax, hmax), inc=(inc, inc, inc))
    return cr, grid


def perturbed_copy(cr: CrystalData, seed, sigma_ang, a_lat, occ_pm):
    """Target structure for the adjoint workload: displacements sigma and
    occupancies 1 +- occ_pm (uniform)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = cr.pos + rng.normal(0.0, 1.0, size=cr.pos.shape) * (sigma_ang / a_lat)
    pos = pos.astype(np.float32).astype(np.float64)
    aocc = (1.0 + rng.uniform(-occ_pm, occ_pm, size=cr.natoms)).astype(np.float32)
    return cr.with_positions(pos, aocc)


def population(seed=5, count=64, nmin=2000, nmax=200000):
    """Batched population: cubic / fcc / rock-salt crystals, atom counts
    log-uniform in [nmin, nmax], each with a 2D plane of 129^2..257^2 points,
    vacancy fraction U(0,0.3), sigma U(0.005,0.05) A, FP32 coordinates."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    kinds = ["cubic", "fcc", "rocksalt"]
    for c in range(count):
        kind = kinds[int(rng.integers(0, 3))]
        target = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        if kind == "cubic":
            a, sites, types = 4.0, [[0, 0, 0], [0.5, 0.5, 0.5]], [1, 2]
        elif kind == "fcc":
            a, sites, types = 3.6, [[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]], [1, 2, 1, 2]
        else:
            fcc = [[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]]
            a = 5.64
            sites = fcc + [[(x + 0.5) % 1.0, y, z] for x, y, z in fcc]
            types = [1] * 4 + [2] * 4
        ncell = max(1, int(round((target / len(sites)) ** (1.0 / 3.0))))
        icc = (ncell, ncell, ncell)
        sigma = rng.uniform(0.005, 0.05)
        vac = rng.uniform(0.0, 0.3)
        pos, iscat = build_periodic(sites, types, icc, a, rng, sigma, fp32=True)
        iscat = np.where(rng.random(iscat.shape[0]) < vac, 0, iscat).astype(np.int32)
        scat, occ, dw = random_form_factors(rng, 2, b_iso=0.5)
        n = int(rng.integers(129, 258))
        n = n if n % 2 == 1 else n + 1
        n = min(n, 257)
        hmax = float(rng.uniform(2.0, 6.0))
        cr = CrystalData(pos=pos, iscat=iscat, nscat=2, ncatoms=len(sites), icc=icc,
                         rten=reciprocal_metric(a, a, a, 90, 90, 90), scat=scat, occ=occ, dw=dw,
                         name=f"pop{c}-{kind}")
        grid = GridData.from_corners((-hmax, -hmax, 0), (hmax, -hmax, 0), (-hmax, hmax, 0), inc=(n, n, 1))
        out.append((cr, grid))
    return out


def small_random(seed=0, natoms=64, nscat=2, inc=(9, 7, 3), span=3.0):
    """Tiny random crystal and 3D grid for unit tests."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pos = rng.uniform(-span, span, size=(natoms, 3))
    iscat = rng.integers(0, nscat + 1, size=natoms).astype(np.int32)
    scat, occ, dw = random_form_factors(rng, nscat, b_iso=0.7)
    grid = GridData(eck=np.array([[-1.3, 1.1, -1.3, -1.3], [-0.9, -0.9, 0.8, -0.9], [-0.5, -0.5, -0.5, 0.4]]),
                    vi=np.array([[0.3, 0.02, 0.01], [0.015, 0.28, -0.02], [0.01, 0.03, 0.45]]),
                    inc=inc)
    cr = CrystalData(pos=pos, iscat=iscat, nscat=nscat, ncatoms=1, icc=(natoms, 1, 1),
                     rten=reciprocal_metric(4.1, 4.3, 5.2, 88, 92, 95), scat=scat, occ=occ, dw=dw,
                     name="small-random")
    return cr, grid


def small_lots_anis(seed=7, icc=(5, 4, 3), nextra=4, inc=(13, 11, 5), anis=True, lxray=True):
    """Small orthorhombic crystal (a, b, c = 4.0, 4.5, 5.0 A) for the ADP and
    lot paths: two sites per cell, two types, one VOID site, cell origins from
    dim0 = (-2, -2, -1); with anis, three ADP types (type 1 split over ADPs 1
    and 3); nextra interstitial atoms stored after the periodic block (the
    atoms four_getatm places in lots by INT(pos)).  The grid is centred on 0
    with odd counts, so Friedel halving applies."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a_lat = np.array([4.0, 4.5, 5.0])
    dim0 = (-2.0, -2.0, -1.0)
    sites = [[0.1, 0.2, 0.3], [0.55, 0.45, 0.6]]
    pos, iscat = build_periodic(sites, [1, 2], icc, a_lat, rng, sigma_ang=0.05)
    pos = pos + np.asarray(dim0)
    iscat[rng.integers(0, iscat.shape[0])] = 0
    ncell = int(np.prod(icc))
    if nextra:
        cells = rng.integers(0, ncell, size=nextra)
        cx = np.stack([cells % icc[0], (cells // icc[0]) % icc[1], cells // (icc[0] * icc[1])], axis=1)
        extra = cx + np.asarray(dim0) + rng.uniform(0.05, 0.95, size=(nextra, 3))
        pos = np.concatenate([pos, extra])
        iscat = np.concatenate([iscat, rng.integers(1, 3, size=nextra).astype(np.int32)])
    scat, occ, dw = random_form_factors(rng, 2, b_iso=0.6)
    occ[1:] = [0.9, 0.75]
    if not lxray:
        scat[:, 1:] = 0.0
    cr = CrystalData(pos=pos, iscat=iscat.astype(np.int32), nscat=2, ncatoms=2, icc=icc,
                     rten=reciprocal_metric(*a_lat, 90, 90, 90), scat=scat, occ=occ, dw=dw, dim0=dim0,
                     ar=tuple(1.0 / a_lat), name="small-lots-anis")
    if anis:
        ianis = np.where(iscat == 2, 2, 1).astype(np.int32)
        ianis[(iscat == 1) & (rng.random(iscat.shape[0]) < 0.4)] = 3
        U = np.array([[0.010, 0.014, 0.008, 0.002, -0.001, 0.003],
                      [0.020, 0.012, 0.016, -0.003, 0.002, 0.001],
                      [0.006, 0.006, 0.006, 0.0, 0.0, 0.0]])
        cr.ianis = ianis
        cr.anis_full = U
    lo = np.array([-1.2, -1.0, -0.8])
    vi = np.diag([2.4 / (inc[0] - 1), 2.0 / (inc[1] - 1), 1.6 / (inc[2] - 1)])
    vi[0, 1] = 0.03
    vi[1, 0] = -0.02
    eck = np.stack([lo, lo + vi[:, 0] * (inc[0] - 1), lo + vi[:, 1] * (inc[1] - 1), lo + vi[:, 2] * (inc[2] - 1)],
                   axis=1)
    # the corners must sum to 0 for Friedel: shift ll so that ll + (n-1) v = -ll
    far = eck[:, 0] + vi @ (np.asarray(inc) - 1)
    eck[:, 0] = eck[:, 0] - (eck[:, 0] + far) / 2
    eck[:, 1] = eck[:, 0] + vi[:, 0] * (inc[0] - 1)
    eck[:, 2] = eck[:, 0] + vi[:, 1] * (inc[1] - 1)
    eck[:, 3] = eck[:, 0] + vi[:, 2] * (inc[2] - 1)
    grid = GridData(eck=eck, vi=vi, inc=inc)
    return cr, grid
