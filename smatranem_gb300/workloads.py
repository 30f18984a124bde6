"""Synthetic structures in the form the SMatrAnEM mesher chain hands the FDTD.

The reference FDTD reads, per cell and component, the complex mu and epsi that
Med3D -> BindData -> CorrF -> PMLgen leave in the Med files: material value
times the metric factor fx_c = H_{c+1} H_{c+2} / H_c (H_j = du_j/dxi_j * h_j,
MixedData/BindData.c:223-228), times the PML stretch s_{c+1} s_{c+2} / s_c
with s = 1 + i*sigma (PMLset/PMLcalc.c:227-231), sigma graded as
sigma_max * |depth/thickness|^p, sigma_max = -(p+1) ln(sqRef) / (4 omega d)
(PMLset/PMLcalc.c:246-260).  The CFL bound written into each Med header is
sqrt(min over cells of e00 e11 e22 m00 m11 m22 / ((e00+e11+e22)(m00+m11+m22)))
(PMLset/PMLcalc.c:279-313); the FDTD takes min_Dt as its square root.

Everything here is seeded numpy; no dataset is involved.  The generators
are plain numpy and load no native code: only prepare(), Prepared.coefficients()
and port_modes() call into the CUDA library (imported where they run), so a
process that must not load it (a CPU-only timing worker) can still build the
structures.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class Structure:
    L: tuple            # (L0, L1, L2, L3)
    mu: np.ndarray      # complex (n3, 3): stretched, as read from the Med files
    epsi: np.ndarray
    omega: float        # k/k0
    min_dt: float       # the FDTD's min_Dt (sqrt of the Med-header "min Dt^2")
    iBc: tuple = (1, 1, 1)
    pec: np.ndarray | None = None  # uint8 (n3,), E coefficients forced to 0
    name: str = ""

    @property
    def n3(self):
        return self.L[0] * self.L[1] * self.L[2]


@dataclasses.dataclass
class Prepared:
    """Outputs of the reference precompute (main :62-143)."""
    s: Structure
    sigma: np.ndarray
    mu: np.ndarray      # after remove_sigma, complex (n3*3,)
    epsi: np.ndarray
    cont: np.ndarray
    addr: np.ndarray
    lnotn: int
    n2pi: int
    invtau_R: float
    invtau_I: float

    def coefficients(self):
        from . import fdtd
        return fdtd.coefficients(self.s.L, self.lnotn, self.sigma, self.mu, self.epsi, self.cont, self.addr,
                                 self.invtau_R, self.invtau_I)

    @property
    def dt(self):
        return 2 * math.pi / (self.s.omega * self.n2pi)


def pml_sigma(n: int, lo: int, hi: int, omega: float, thick_lo: float, thick_hi: float,
              sq_ref: float = 1e-12, power: int = 3):
    """sigma at the H (h=0) and E (h=1) sub-points of n cells with lo/hi PML cells.

    The H sub-point of cell j sits at j + 0.5 and the E sub-point at j + 1.0 in
    cell units (the E component is half a cell forward of H along its own axis,
    as the forward difference ope_R implies)."""
    out = np.zeros((2, n))
    for h, shift in ((0, 0.5), (1, 1.0)):
        x = np.arange(n) + shift
        if lo > 0:
            smax = -(power + 1) * math.log(sq_ref) / (4 * omega * thick_lo)
            d = np.clip((lo - x) / lo, 0, None)
            out[h] += smax * d ** power
        if hi > 0:
            smax = -(power + 1) * math.log(sq_ref) / (4 * omega * thick_hi)
            d = np.clip((x - (n - hi)) / hi, 0, None)
            out[h] += smax * d ** power
    return out


def sigma_vector(L, sig_axes):
    """Pack per-axis (2, L_a) profiles into the reference's 2*(L0+L1+L2) layout."""
    parts = []
    for a in range(3):
        s = sig_axes[a]
        v = np.zeros(2 * L[a])
        v[0::2] = s[0]
        v[1::2] = s[1]
        parts.append(v)
    return np.concatenate(parts)


def stretch_media(L, mu_r, eps_r, sig_axes):
    """Apply the PMLgen stretch: mu_c *= s_h(c+1) s_h(c+2) / s_e(c), epsi swapped."""
    L0, L1, L2 = L[:3]
    j = np.indices((L2, L1, L0)).reshape(3, -1)[::-1]  # j[0] fastest
    s = []
    for h in range(2):
        s.append([1 + 1j * sig_axes[a][h][j[a]] for a in range(3)])
    mu = np.array(mu_r, dtype=np.complex128, copy=True)
    ep = np.array(eps_r, dtype=np.complex128, copy=True)
    for c in range(3):
        a1, a2 = (c + 1) % 3, (c + 2) % 3
        mu[:, c] *= s[0][a1] * s[0][a2] / s[1][c]
        ep[:, c] *= s[1][a1] * s[1][a2] / s[0][c]
    return mu, ep


def cfl_min_dt(mu_r, eps_r):
    """min_Dt of the FDTD from real media (PMLcalc.c:279-313 then sqrt)."""
    m = np.real(mu_r)
    e = np.real(eps_r)
    r = (e[:, 0] * e[:, 1] * e[:, 2] * m[:, 0] * m[:, 1] * m[:, 2]) / (e.sum(1) * m.sum(1))
    r = r[np.isfinite(r) & (r > 0)]
    return math.sqrt(math.sqrt(r.min()))


def metric_fx(Hs):
    """fx_c = H_{c+1} H_{c+2} / H_c from per-cell scale factors Hs (n3, 3)."""
    fx = np.empty_like(Hs)
    for c in range(3):
        fx[:, c] = Hs[:, (c + 1) % 3] * Hs[:, (c + 2) % 3] / Hs[:, c]
    return fx


def random_structure(L, seed=0, pml=(2, 2, 2), pml_z_only=False, metals=0.0, lossy=0.0, pec=0.0,
                     iBc=(1, 1, 1), omega=0.4, dx=0.2, aniso=0.15, sq_ref=1e-8):
    """A small seeded structure exercising every cell class of the reference.

    metals/lossy/pec are fractions of interior cells (outside the PML and off
    the centre lines the FDTD reads sigma from) that become 'e'/'h'/'b' cells,
    absorbing dielectrics, or PEC cells.  A metal component gets a Drude-like
    epsi (Re < 0, Im > 0) or a mu with Re > 0, Im < 0; both have tan(arg) < 0,
    the reference's test for its stable-form update.  That update is not
    unconditionally stable (fields near such cells can grow), so tests that use
    metals run few steps."""
    rng = np.random.default_rng(seed)
    L0, L1, L2, L3 = L
    n3 = L0 * L1 * L2
    Hs = dx * rng.uniform(1 - aniso, 1 + aniso, size=(n3, 3))
    fx = metric_fx(Hs)
    mu_r = fx * rng.uniform(0.9, 1.3, size=(n3, 3))
    eps_r = fx * rng.uniform(1.0, 6.0, size=(n3, 3))
    min_dt = cfl_min_dt(mu_r, eps_r)
    j = np.indices((L2, L1, L0)).reshape(3, -1)[::-1]
    p = pml
    thick = [p[a] * dx for a in range(3)]
    sig = []
    for a, n in enumerate((L0, L1, L2)):
        if pml_z_only and a < 2:
            sig.append(np.zeros((2, n)))
        else:
            sig.append(pml_sigma(n, p[a], p[a], omega, max(thick[a], 1e-9), max(thick[a], 1e-9), sq_ref))
    interior = np.ones(n3, bool)
    for a, n in enumerate((L0, L1, L2)):
        if not (pml_z_only and a < 2):
            interior &= (j[a] >= p[a] + 1) & (j[a] < n - p[a] - 1)
    # keep the centre lines the FDTD reads sigma from clean
    c0, c1, c2 = L0 // 2, L1 // 2, L2 // 2
    on_line = ((j[1] == c1) & (j[2] == c2)) | ((j[0] == c0) & (j[2] == c2)) | ((j[0] == c0) & (j[1] == c1))
    cand = np.flatnonzero(interior & ~on_line)
    rng.shuffle(cand)
    nm, nl, npc = (int(round(f * len(cand))) for f in (metals, lossy, pec))
    mcells, lcells, pcells = cand[:nm], cand[nm:nm + nl], cand[nm + nl:nm + nl + npc]
    mu_c = mu_r.astype(np.complex128)
    ep_c = eps_r.astype(np.complex128)
    for i, l in enumerate(mcells):
        kind = i % 3  # 'e', 'h', 'b'
        comp = rng.integers(0, 3)
        if kind in (0, 2):
            ep_c[l, comp] = fx[l, comp] * (-rng.uniform(2, 20) + 1j * rng.uniform(0.5, 3))
        if kind in (1, 2):
            mu_c[l, comp] = fx[l, comp] * (rng.uniform(1, 2) - 1j * rng.uniform(0.1, 1))
    for l in lcells:
        ep_c[l] += 1j * fx[l] * rng.uniform(0.01, 0.5, size=3)
    mu_s, ep_s = stretch_media(L, mu_c, ep_c, sig)
    pec_mask = None
    if npc:
        pec_mask = np.zeros(n3, np.uint8)
        pec_mask[pcells] = 1
    return Structure(L=tuple(L), mu=mu_s, epsi=ep_s, omega=omega, min_dt=min_dt, iBc=tuple(iBc), pec=pec_mask,
                     name=f"random{tuple(L)}")


def prepare(s: Structure, dt_factor: float = 1.0) -> Prepared:
    """The reference precompute through the library (set_sigma .. set_tau)."""
    from . import fdtd
    mu = np.ascontiguousarray(s.mu.reshape(-1))
    ep = np.ascontiguousarray(s.epsi.reshape(-1))
    sigma = fdtd.set_sigma(s.L, mu, ep)
    mu2, ep2 = fdtd.remove_sigma(s.L, mu, ep, sigma)
    cont, addr, lnotn = fdtd.set_address(s.L, sigma, mu2, ep2)
    n2pi, iR, iI = fdtd.set_tau(s.omega, s.min_dt / dt_factor)
    return Prepared(s=s, sigma=sigma, mu=mu2, epsi=ep2, cont=cont, addr=addr, lnotn=lnotn, n2pi=n2pi,
                    invtau_R=iR, invtau_I=iI)


def random_fields(n, lnotn, seed=0, scale=1.0):
    """Random H_t, E_t in the reference layout (sentinel zero)."""
    rng = np.random.default_rng(seed)
    m = 3 * (n + lnotn + 1)
    H = rng.standard_normal(m) * scale
    E = rng.standard_normal(m) * scale
    H[-3:] = 0
    E[-3:] = 0
    return H, E


def random_incident(pl, seed=0, real_e=True):
    rng = np.random.default_rng(seed)
    Hinc = rng.standard_normal(2 * pl) + 1j * rng.standard_normal(2 * pl)
    Einc = rng.standard_normal(2 * pl) + (0 if real_e else 1j * rng.standard_normal(2 * pl))
    return Hinc.astype(np.complex128), np.asarray(Einc, dtype=np.complex128)


# ---------------------------------------------------------------------------
# Curvilinear strip-waveguide bend (the bend benchmark structure)
# ---------------------------------------------------------------------------

INV_K0_UM = 0.1  # unit of length: 1/k0 = 0.1 um, as in the reference example deck


def graded_spacing(n, center, fine, coarse, width):
    """Cell sizes growing smoothly from `fine` at cell `center` to `coarse`."""
    d = np.arange(n) + 0.5 - center
    return fine + (coarse - fine) * (1.0 - np.exp(-(d / width) ** 2))


@dataclasses.dataclass
class Bend:
    s: Structure
    iB: int
    iT: int
    iI: int
    pml: int
    u0: np.ndarray   # cell-centre coordinates across (um), core centre at 0
    u1: np.ndarray
    n_eff: float = 2.4
    port_med: np.ndarray | None = None  # (6, L0*L1) lossless Med values of a port layer (before the PML stretch)


def bend_structure(shape=(256, 192, 160), pml=12, L3=16, radius_um=2.0, core=(0.45, 0.22), eps_core=12.11,
                   eps_clad=2.085, lam0_um=1.55, cell_um=(0.015, 0.025), core_cell0=45, dt_factor=1.0 / 0.99,
                   sq_ref=1e-12, power=3) -> Bend:
    """Silicon strip 90-degree bend in orthogonal curvilinear coordinates.

    u0 is the in-plane transverse (radial) coordinate, u1 the vertical one and
    u2 the arc length along the bend; the bend (curvature 1/R) spans the
    L2 - 2*L3 scatterer layers and the L3 outer layers at each end are straight
    ports.  Metric: H0 = du0, H1 = du1, H2 = du2 * (1 + kappa*u0) (the scale
    factor of polar coordinates), fx_c = H_{c+1} H_{c+2} / H_c per cell, so
    every cell carries distinct coefficients.  Cell sizes du0, du1 grade from
    15 nm at the core to 25 nm; du2 = quarter-circle length / bend layers.  The
    core sits near the inner side of the bend (cell core_cell0 of L0) so that
    1 + kappa*u0 stays above 0.5.  12-cell split PML on all six faces."""
    L0, L1, L2 = shape
    L3 = min(L3, max(pml + 3, L2 // 4))
    fine, coarse = (c / INV_K0_UM for c in cell_um)
    du0 = graded_spacing(L0, core_cell0, fine, coarse, 40.0)
    du1 = graded_spacing(L1, L1 / 2, fine, coarse, 30.0)
    u0 = np.cumsum(du0) - 0.5 * du0
    u0 = u0 - u0[core_cell0]
    u1 = np.cumsum(du1) - 0.5 * du1
    u1 = u1 - u1[L1 // 2]
    R = radius_um / INV_K0_UM
    nb = L2 - 2 * L3
    du2 = np.full(L2, fine + 0.25 * (coarse - fine))
    du2[L3:L2 - L3] = 0.5 * math.pi * R / nb
    kappa = np.zeros(L2)
    kappa[L3:L2 - L3] = 1.0 / R
    omega = 2 * math.pi * INV_K0_UM / lam0_um
    n3 = L0 * L1 * L2
    j0 = np.tile(np.arange(L0), L1 * L2)
    j1 = np.tile(np.repeat(np.arange(L1), L0), L2)
    j2 = np.repeat(np.arange(L2), L0 * L1)
    h2 = 1.0 + kappa[j2] * u0[j0]
    Hs = np.stack([du0[j0], du1[j1], du2[j2] * h2], axis=1)
    fx = metric_fx(Hs)
    del Hs, h2
    in_core = (np.abs(u0[j0]) <= 0.5 * core[0] / INV_K0_UM) & (np.abs(u1[j1]) <= 0.5 * core[1] / INV_K0_UM)
    eps_r = np.where(in_core, eps_core, eps_clad)[:, None] * fx
    mu_r = fx
    min_dt = cfl_min_dt(mu_r, eps_r) / dt_factor * dt_factor  # header value; dt_factor applied in set_tau
    sig = []
    for a, (n, d) in enumerate(((L0, du0), (L1, du1), (L2, du2))):
        th_lo, th_hi = float(d[:pml].sum()), float(d[n - pml:].sum())
        sig.append(pml_sigma(n, pml, pml, omega, th_lo, th_hi, sq_ref, power))
    mu_s, ep_s = stretch_media((L0, L1, L2), mu_r, eps_r, sig)
    pl = L0 * L1
    zi = min(pml + 3, L3 - 1)  # a straight port layer (every port layer has the same media)
    m_l, e_l = mu_r[zi * pl:(zi + 1) * pl], eps_r[zi * pl:(zi + 1) * pl]
    port_med = np.stack([m_l[:, 0], m_l[:, 1], e_l[:, 2], e_l[:, 1], e_l[:, 0], m_l[:, 2]]).astype(np.complex128)
    del mu_r, eps_r, fx
    s = Structure(L=(L0, L1, L2, L3), mu=mu_s, epsi=ep_s, omega=omega, min_dt=min_dt, iBc=(0, 0, 0),
                  name=f"bend{L0}x{L1}x{L2}")
    return Bend(s=s, iB=pml + 1, iT=L2 - pml - 2, iI=pml + 3, pml=pml, u0=u0 * INV_K0_UM, u1=u1 * INV_K0_UM,
                port_med=port_med)


def mode_profiles(b: Bend, n_modes=4, w0_um=0.26, w1_um=0.16):
    """Approximate guided-mode sheets of the strip: TE0, TM0, TE1, TM1.

    Returns a list of (Hinc, Einc) complex planes (2*L0*L1, component v of pixel
    p at v + 2p) for propagation along +u2: TE modes carry E_x with
    H_y = n_eff E_x, TM modes E_y with H_x = -n_eff E_y.  Normalised to unit
    overlap norm.  Stand-ins for the port eigenmodes where only the update
    rate matters; port_modes() gives the eigenmodes themselves."""
    L0, L1 = b.s.L[0], b.s.L[1]
    x = b.u0[None, :] / w0_um
    y = b.u1[:, None] / w1_um
    g = np.exp(-x ** 2 - y ** 2)
    shapes = [g, g, x * g, y * g]
    out = []
    for m in range(n_modes):
        f = shapes[m].reshape(-1)
        f = f / math.sqrt(2 * b.n_eff * float(np.sum(f * f)))
        Hinc = np.zeros(2 * L0 * L1, np.complex128)
        Einc = np.zeros(2 * L0 * L1, np.complex128)
        if m % 2 == 0:  # TE: E_x, H_y
            Einc[0::2] = f
            Hinc[1::2] = b.n_eff * f
        else:           # TM: E_y, H_x
            Einc[1::2] = f
            Hinc[0::2] = -b.n_eff * f
        out.append((Hinc, Einc))
    return out


def port_modes(b: Bend, n_modes=4, **solve_kw):
    """The first n_modes propagating eigenmodes of the bend's port layer
    (lossless media with their metric factors, PEC box) from the GPU mode
    solver: a modes.Modes with Mcalc's theta and Xi columns."""
    from . import modes as M
    return M.solve(b.port_med, b.s.omega, b.s.L[0], b.s.L[1], b.s.iBc[:2], n_modes, **solve_kw)


def pulse_schedule(nsteps, dt, lam0_um=1.55, bandwidth=0.2, lams_um=None, delay_sigmas=4.0):
    """Gaussian-modulated sine sheet source and DFT phases at wavelengths lams_um.

    Source: g(t) sin(omega0 t) with g a Gaussian whose spectral FWHM is
    `bandwidth` * omega0; E sheets at t = (k+1/2) dt, H sheets at (k+1) dt (the
    reference's half-step times).  DFT weights exp(i omega t) at the same times
    as the reference's ExpN (main :93-99, :165)."""
    w0 = 2 * math.pi * INV_K0_UM / lam0_um
    sigma_w = bandwidth * w0 / 2.355
    tau = 1.0 / sigma_w
    t0 = delay_sigmas * tau
    k = np.arange(nsteps)
    tE, tH = (k + 0.5) * dt, (k + 1.0) * dt
    src = np.zeros((nsteps, 6))
    src[:, 0] = np.exp(-0.5 * ((tE - t0) / tau) ** 2)
    src[:, 1] = np.sin(w0 * tE)
    src[:, 3] = np.exp(-0.5 * ((tH - t0) / tau) ** 2)
    src[:, 4] = np.sin(w0 * tH)
    if lams_um is None:
        lams_um = [lam0_um]
    om = 2 * math.pi * INV_K0_UM / np.asarray(lams_um, dtype=np.float64)
    ph = np.empty((nsteps, len(om), 4))
    ph[:, :, 0] = np.cos(om[None] * tH[:, None])
    ph[:, :, 1] = np.sin(om[None] * tH[:, None])
    ph[:, :, 2] = np.cos(om[None] * (tH[:, None] + 0.5 * dt))
    ph[:, :, 3] = np.sin(om[None] * (tH[:, None] + 0.5 * dt))
    return src, ph


def overlap(dft_plane, Hinc, Einc):
    """Mode overlap of one DFT plane (4, pl: Hx, Hy, Ex, Ey) with a mode sheet:
    sum conj(mode) . (Hx, Hy, -Ey, Ex), the vector S_calc projects
    (FDTDsplitfieldMetal.c:437-445) with the mode in the same arrangement."""
    mh = np.stack([Hinc[0::2], Hinc[1::2]])
    me = np.stack([-Einc[1::2], Einc[0::2]])
    v = np.stack([dft_plane[0], dft_plane[1], -dft_plane[3], dft_plane[2]])
    m = np.concatenate([mh, me])
    return complex(np.sum(np.conj(m) * v))


# ---------------------------------------------------------------------------
# Inverse-design structure (the adjoint-gradient workload)
# ---------------------------------------------------------------------------

@dataclasses.dataclass
class Design(Bend):
    box: tuple = (0, 0, 0, 0, 0, 0)   # design cells [x0, x1) x [y0, y1) x [z0, z1)
    eps: np.ndarray | None = None     # their eps_r, (nz, ny, nx)
    eps_base: np.ndarray | None = None  # stretched epsi of the whole grid, design cells at eps_r = 1

    def with_eps(self, eps) -> Structure:
        """The structure with design permittivities eps (nz, ny, nx); the
        design box lies outside the PML, so a cell's stored epsi is eps_r times
        the metric factor dx (held in eps_base)."""
        x0, x1, y0, y1, z0, z1 = self.box
        L0, L1 = self.s.L[0], self.s.L[1]
        ep = self.eps_base.copy()
        j = np.indices((z1 - z0, y1 - y0, x1 - x0)).reshape(3, -1)
        cells = (x0 + j[2]) + L0 * ((y0 + j[1]) + L1 * (z0 + j[0]))
        ep[cells, :] = self.eps_base[cells, :] * np.asarray(eps, dtype=np.float64).reshape(-1)[:, None]
        return dataclasses.replace(self.s, epsi=ep)


def design_structure(shape=(160, 160, 120), design=(60, 60, 20), pml=12, seed=0, core=(0.45, 0.22),
                     eps_core=12.11, eps_clad=2.085, eps_range=(2.085, 12.11), dx_um=0.02, lam0_um=1.55,
                     sq_ref=1e-12, power=3, pml_xy=True) -> Design:
    """A straight silicon strip along z (two single-mode ports) through a
    design region of seeded random permittivity, on a uniform grid of dx_um
    cells (metric factor dx), split PML on all six faces (pml_xy=False: on the
    z faces only, x/y walls with iBc = 0, so that the monitor planes hold no
    PML cell and the reference's own DFT applies).  Source plane iI and
    monitor planes iB (below the source) and iT (the output port, above the
    design region)."""
    L0, L1, L2 = shape
    nx, ny, nz = design
    dx = dx_um / INV_K0_UM
    n3 = L0 * L1 * L2
    u0 = (np.arange(L0) + 0.5 - 0.5 * L0) * dx_um
    u1 = (np.arange(L1) + 0.5 - 0.5 * L1) * dx_um
    j = np.indices((L2, L1, L0)).reshape(3, -1)[::-1]
    in_core = (np.abs(u0[j[0]]) <= 0.5 * core[0]) & (np.abs(u1[j[1]]) <= 0.5 * core[1])
    eps_r = np.where(in_core, eps_core, eps_clad)
    x0, y0, z0 = (L0 - nx) // 2, (L1 - ny) // 2, (L2 - nz) // 2
    box = (x0, x0 + nx, y0, y0 + ny, z0, z0 + nz)
    in_box = (j[0] >= x0) & (j[0] < x0 + nx) & (j[1] >= y0) & (j[1] < y0 + ny) & (j[2] >= z0) & (j[2] < z0 + nz)
    rng = np.random.default_rng(seed)
    eps_d = rng.uniform(eps_range[0], eps_range[1], size=(nz, ny, nx))
    eps_r = np.where(in_box, 1.0, eps_r)
    # metric factor fx_c = H_{c+1} H_{c+2} / H_c = dx on a uniform grid
    mu_r = np.full((n3, 3), dx)
    eps3 = np.repeat(eps_r[:, None] * dx, 3, axis=1)
    omega = 2 * math.pi * INV_K0_UM / lam0_um
    sig = [pml_sigma(n, pml, pml, omega, pml * dx, pml * dx, sq_ref, power) if (a == 2 or pml_xy)
           else np.zeros((2, n)) for a, n in enumerate((L0, L1, L2))]
    mu_s, ep_s = stretch_media((L0, L1, L2), mu_r, eps3, sig)
    eps_min = np.full((n3, 3), min(eps_clad, eps_range[0]) * dx)
    min_dt = cfl_min_dt(mu_r, eps_min)
    s = Structure(L=(L0, L1, L2, pml + 2), mu=mu_s, epsi=ep_s, omega=omega, min_dt=min_dt, iBc=(0, 0, 0),
                  name=f"design{L0}x{L1}x{L2}")
    d = Design(s=s, iB=pml + 1, iT=L2 - pml - 2, iI=pml + 3, pml=pml, u0=u0, u1=u1, box=box, eps=eps_d,
               eps_base=ep_s)
    d.s = d.with_eps(eps_d)
    return d


@dataclasses.dataclass
class Cube:
    s: Structure
    iI: int          # source plane (the point source sits at pixel src_px of it)
    iM: int          # monitor plane of the running DFT
    src_px: int      # j0 + L0*j1 of the point source
    pml: int


def cube_structure(n=96, pml=10, cube=30, plate=40, gap=15, eps_cube=12.11, dx_um=0.02, lam0_um=1.55,
                   reflection=1e-6, power=3) -> Cube:
    """The plain FP64 benchmark case: n^3 uniform cells of dx_um in vacuum
    (metric factor dx), a centred cube^3 dielectric block of eps_cube, a
    one-cell-thick plate x plate PEC plate `gap` cells below the block, split
    PML of `pml` cells on all six faces (polynomial grading `power`, normal
    reflection `reflection`: the PML deck's squareRef is its square).  An x
    point source (one pixel of the sheet source, driving E_x) on a plane above
    the block; the monitor plane between the plate and the block."""
    L0 = L1 = L2 = n
    dx = dx_um / INV_K0_UM
    n3 = n ** 3
    j = np.indices((L2, L1, L0)).reshape(3, -1)[::-1]
    c0 = (n - cube) // 2
    in_cube = np.all([(j[a] >= c0) & (j[a] < c0 + cube) for a in range(3)], axis=0)
    eps_r = np.where(in_cube, eps_cube, 1.0)
    mu_r = np.full((n3, 3), dx)
    eps3 = np.repeat(eps_r[:, None] * dx, 3, axis=1)
    omega = 2 * math.pi * INV_K0_UM / lam0_um
    sig = [pml_sigma(n, pml, pml, omega, pml * dx, pml * dx, reflection ** 2, power) for _ in range(3)]
    mu_s, ep_s = stretch_media((L0, L1, L2), mu_r, eps3, sig)
    min_dt = cfl_min_dt(mu_r, np.full((n3, 3), dx))
    zp, p0 = c0 - gap, (n - plate) // 2
    pec = ((j[2] == zp) & (j[0] >= p0) & (j[0] < p0 + plate) & (j[1] >= p0) & (j[1] < p0 + plate)).astype(np.uint8)
    s = Structure(L=(L0, L1, L2, pml + 2), mu=mu_s, epsi=ep_s, omega=omega, min_dt=min_dt, iBc=(0, 0, 0), pec=pec,
                  name=f"cube{n}")
    iI = c0 + cube + (L2 - pml - (c0 + cube)) // 2
    iM = zp + (c0 - zp) // 2
    return Cube(s=s, iI=iI, iM=iM, src_px=n // 2 + L0 * (n // 2), pml=pml)


def point_source(c: Cube):
    """Sheet arrays (Hinc, Einc, 2*L0*L1 complex each) of the x point source:
    the H-sheet component that drives E_x (W_0 += s * Hi_1 in the E step,
    main_calc :293-296) is 1 at the source pixel, everything else 0."""
    pl = c.s.L[0] * c.s.L[1]
    Hinc = np.zeros(2 * pl, np.complex128)
    Einc = np.zeros(2 * pl, np.complex128)
    Hinc[1 + 2 * c.src_px] = 1.0
    return Hinc, Einc


def slab_structure(shape, seed=0, pml=12, slab_um=0.22, eps_slab=12.11, eps_clad=2.085,
                   eps_range=(2.085, 12.11), n_incl=(1, 6), dx_um=0.02, lam0_um=1.55, sq_ref=1e-12,
                   power=3) -> Bend:
    """A silicon slab (normal to y) in SiO2 with 1-6 seeded cuboid inclusions of
    random permittivity, on a uniform grid of dx_um cells, split PML on all six
    faces.  Returned as a Bend-like record (source plane iI, monitor planes iB,
    iT) so that mode_profiles() gives its port sheets."""
    L0, L1, L2 = shape
    dx = dx_um / INV_K0_UM
    n3 = L0 * L1 * L2
    rng = np.random.default_rng(seed)
    u0 = (np.arange(L0) + 0.5 - 0.5 * L0) * dx_um
    u1 = (np.arange(L1) + 0.5 - 0.5 * L1) * dx_um
    j = np.indices((L2, L1, L0)).reshape(3, -1)[::-1]
    eps_r = np.where(np.abs(u1[j[1]]) <= 0.5 * slab_um, eps_slab, eps_clad).astype(np.float64)
    lo, hi = pml + 2, [n - pml - 2 for n in (L0, L1, L2)]
    for _ in range(int(rng.integers(n_incl[0], n_incl[1] + 1))):
        a = [int(rng.integers(lo, max(lo + 1, hi[d] - 8))) for d in range(3)]
        b = [min(hi[d], a[d] + int(rng.integers(4, max(5, (hi[d] - lo) // 3)))) for d in range(3)]
        inside = np.ones(n3, bool)
        for d in range(3):
            inside &= (j[d] >= a[d]) & (j[d] < b[d])
        eps_r[inside] = rng.uniform(*eps_range)
    mu_r = np.full((n3, 3), dx)
    eps3 = np.repeat(eps_r[:, None] * dx, 3, axis=1)
    omega = 2 * math.pi * INV_K0_UM / lam0_um
    sig = [pml_sigma(n, pml, pml, omega, pml * dx, pml * dx, sq_ref, power) for n in (L0, L1, L2)]
    mu_s, ep_s = stretch_media((L0, L1, L2), mu_r, eps3, sig)
    min_dt = cfl_min_dt(mu_r, np.full((n3, 3), min(eps_clad, eps_range[0]) * dx))
    s = Structure(L=(L0, L1, L2, pml + 2), mu=mu_s, epsi=ep_s, omega=omega, min_dt=min_dt, iBc=(0, 0, 0),
                  name=f"slab{L0}x{L1}x{L2}")
    return Bend(s=s, iB=pml + 1, iT=L2 - pml - 2, iI=pml + 3, pml=pml, u0=u0, u1=u1)


def slab_shapes(n=16, seed=0, lo=(128, 128, 128), hi=(256, 256, 192)):
    """n seeded grid shapes from lo to hi (multiples of 8 in x, for the float4
    sweeps): the uneven structures of the batched S-matrix workload."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        t = i / max(1, n - 1)
        shp = []
        for d in range(3):
            v = lo[d] + t * (hi[d] - lo[d]) + rng.integers(-8, 9)
            v = int(min(hi[d], max(lo[d], v)))
            shp.append(v - v % 8)
        out.append(tuple(shp))
    return out


def large_structure(shape=(640, 640, 512), pml=12, radius_um=50.0, dx_um=0.02, eps_sub=2.085, sub=(0.30, 0.50),
                    period=40, patch=20, thick=2, lam0_um=1.55, beam_um=4.0, sq_ref=1e-12, power=3) -> Bend:
    """Large-domain workload: an eps_sub slab (z fraction `sub` of the grid) in
    vacuum carrying a PEC patch array (patch x patch x thick cells, period
    cells, clipped to the non-PML cells) on its top face, on a gently curved
    substrate: cylindrical coordinates with the x arc at radius R + u2, so
    H0 = dx (1 + (u2 - u2_mid) / R), H1 = H2 = dx.  Split PML on all six
    faces.  Built plane by plane (the grid has ~210M cells); only the
    stretched mu and epsi (complex, n3 x 3) are held in full."""
    L0, L1, L2 = shape
    dx = dx_um / INV_K0_UM
    pl = L0 * L1
    n3 = pl * L2
    omega = 2 * math.pi * INV_K0_UM / lam0_um
    sig = [pml_sigma(n, pml, pml, omega, pml * dx, pml * dx, sq_ref, power) for n in (L0, L1, L2)]
    u2 = (np.arange(L2) + 0.5) * dx_um
    h0 = 1.0 + (u2 - u2.mean()) / radius_um
    z0, z1 = int(sub[0] * L2), int(sub[1] * L2)
    # patch mask of one plane
    jx = np.arange(L0)
    jy = np.arange(L1)
    off = (period - patch) // 2
    px_in = ((jx % period) >= off) & ((jx % period) < off + patch) & (jx >= pml + 1) & (jx < L0 - pml - 1)
    py_in = ((jy % period) >= off) & ((jy % period) < off + patch) & (jy >= pml + 1) & (jy < L1 - pml - 1)
    patch2d = (py_in[:, None] & px_in[None, :]).reshape(-1)
    mu = np.empty((n3, 3), np.complex128)
    ep = np.empty((n3, 3), np.complex128)
    pec = np.zeros(n3, np.uint8)
    # in-plane stretch factors s_h, s_e for x and y (z: per plane)
    sx = [1 + 1j * sig[0][h] for h in range(2)]
    sy = [1 + 1j * sig[1][h] for h in range(2)]
    sxy = [[np.tile(sx[h], L1), np.repeat(sy[h], L0)] for h in range(2)]
    r_min = np.inf
    for z in range(L2):
        fx = np.array([dx / h0[z], dx * h0[z], dx * h0[z]])  # H1 H2 / H0, H2 H0 / H1, H0 H1 / H2
        eps_z = eps_sub if z0 <= z < z1 else 1.0
        m = np.broadcast_to(fx, (pl, 3)).astype(np.complex128)
        e = (eps_z * m).copy()
        sz = [1 + 1j * sig[2][h][z] for h in range(2)]
        s = [[sxy[h][0], sxy[h][1], np.full(pl, sz[h])] for h in range(2)]
        for c in range(3):
            a1, a2 = (c + 1) % 3, (c + 2) % 3
            m[:, c] = m[:, c] * s[0][a1] * s[0][a2] / s[1][c]
            e[:, c] = e[:, c] * s[1][a1] * s[1][a2] / s[0][c]
        mu[z * pl:(z + 1) * pl] = m
        ep[z * pl:(z + 1) * pl] = e
        if z1 <= z < z1 + thick:
            pec[z * pl:(z + 1) * pl] = patch2d
        er, mr = eps_z * fx, fx
        r_min = min(r_min, float(np.prod(er) * np.prod(mr) / (er.sum() * mr.sum())))
    min_dt = math.sqrt(math.sqrt(r_min))
    s = Structure(L=(L0, L1, L2, pml + 2), mu=mu, epsi=ep, omega=omega, min_dt=min_dt, iBc=(0, 0, 0), pec=pec,
                  name=f"large{L0}x{L1}x{L2}")
    u0 = (np.arange(L0) + 0.5 - 0.5 * L0) * dx_um
    u1 = (np.arange(L1) + 0.5 - 0.5 * L1) * dx_um
    # source below the slab, launched towards +z through slab and grating;
    # coordinates scaled so that mode_profiles' Gaussian is beam_um wide
    b = Bend(s=s, iB=pml + 1, iT=L2 - pml - 2, iI=pml + 3, pml=pml, u0=u0 * (2.0 / beam_um),
             u1=u1 * (2.0 / beam_um), n_eff=1.0)
    return b


def port_layer(L0, L1, core=(4, 3), eps_core=12.11, eps_clad=2.085, seed=0, jitter=0.0, metric=0.0, loss=0.0):
    """One synthetic z layer of port media for the mode solver: (6, L0*L1)
    complex values in the Med file's column order (j2 = 0: mu00, mu11, eps22;
    j2 = 1: eps11, eps00, mu22), metric factor included.

    A core of core[0] x core[1] cells with relative permittivity eps_core,
    centred, in eps_clad; jitter perturbs the core permittivity per cell by up
    to that fraction, metric multiplies every value by a seeded factor in
    [1 - metric, 1 + metric] (a non-uniform mesh), loss adds i*loss*eps to the
    core permittivity (lossy media make the eigenproblem complex).  Seeded."""
    rng = np.random.default_rng(seed)
    n = L0 * L1
    j0 = np.tile(np.arange(L0), L1)
    j1 = np.repeat(np.arange(L1), L0)
    c0, c1 = (L0 - core[0]) // 2, (L1 - core[1]) // 2
    in_core = (j0 >= c0) & (j0 < c0 + core[0]) & (j1 >= c1) & (j1 < c1 + core[1])
    eps = np.where(in_core, eps_core, eps_clad).astype(np.complex128)
    if jitter:
        eps = eps * np.where(in_core, 1.0 + jitter * (rng.random(n) - 0.5) * 2.0, 1.0)
    if loss:
        eps = eps + 1j * loss * np.where(in_core, eps.real, 0.0)
    med = np.stack([np.ones(n), np.ones(n), eps, eps, eps, np.ones(n)]).astype(np.complex128)
    if metric:
        med = med * (1.0 + metric * (2.0 * rng.random((6, n)) - 1.0))
    return med


def waveguide_structure(med, L0, L1, L2, L3, omega=0.405, pml_z=3, iBc=(0, 0, 0), sq_ref=1e-8):
    """A straight guide along z: the port layer med ((6, L0*L1), from
    port_layer) repeated on all L2 layers, a split PML of pml_z layers at each
    z end and none across (the port layers stay lossless, as the mesher
    chain's PMLgen leaves them, PMLset/PMLcalc.c:222).  With
    modes.solve(med, omega, L0, L1, iBc[:2]) this is a deck whose incident
    and overlap columns come from the layer's own eigenmodes."""
    med = np.asarray(med, np.complex128).reshape(6, L0 * L1)
    pl = L0 * L1
    mu = np.zeros((L2 * pl, 3), np.complex128)
    ep = np.zeros((L2 * pl, 3), np.complex128)
    mu[:, 0], mu[:, 1], ep[:, 2] = (np.tile(med[k], L2) for k in (0, 1, 2))
    ep[:, 1], ep[:, 0], mu[:, 2] = (np.tile(med[k], L2) for k in (3, 4, 5))
    min_dt = cfl_min_dt(mu.real, ep.real)
    sig = [np.zeros((2, L0)), np.zeros((2, L1)),
           pml_sigma(L2, pml_z, pml_z, omega, float(pml_z), float(pml_z), sq_ref)]
    mu_s, ep_s = stretch_media((L0, L1, L2), mu, ep, sig)
    return Structure(L=(L0, L1, L2, L3), mu=mu_s, epsi=ep_s, omega=omega, min_dt=min_dt, iBc=tuple(iBc),
                     name=f"guide{L0}x{L1}x{L2}")


def plane_wave_basis(L0, L1, eps=2.085, omega=0.405):
    """The full mode matrix Xi of a uniform, isotropic, periodic port layer
    (BoundC = (1, 1), mu = 1, unit cells) in Mcalc's conventions, built in
    closed form instead of by a dense eigen solve.  For wavevector k the
    forward differences have the symbols d_a = e^{i k_a} - 1, maa the
    Hermitian symbol M = w mu - (1/(w eps)) c^H c with c = (d1, -d0), and
    mbb*maa the eigenvalue w^2 eps mu - |d|^2 on both polarizations
    (u1 = c^H / |c| and u2 = (d0, d1) / |d|, eigenvectors of M; e_x, e_y at
    k = 0).  Then Mcalc's steps: eiSin = the root with Im >= 0, theta =
    2 asin(eiSin / 2), E = maa H / eiSin, forward [e^{-i theta/2} H; E] and
    backward [e^{i theta/2} H; -E] columns, propagating modes first by
    descending theta and evanescent ones by ascending Im theta, and normXi's
    normalisations (unit power flow; unit cross flow of an evanescent pair).
    Returns (theta (2N,), Xi (2N, 2N), num_real), N = 2*L0*L1."""
    NA1 = L0 * L1
    N = 2 * NA1
    w = omega
    j0 = np.tile(np.arange(L0), L1)
    j1 = np.repeat(np.arange(L1), L0)
    modes = []
    for q in range(L1):
        for p in range(L0):
            k0, k1 = 2 * math.pi * p / L0, 2 * math.pi * q / L1
            d0, d1 = np.exp(1j * k0) - 1, np.exp(1j * k1) - 1
            c = np.array([d1, -d0])
            M = w * np.eye(2) - np.outer(np.conj(c), c) / (w * eps)
            lam = w * w * eps - (abs(d0) ** 2 + abs(d1) ** 2)
            ph = np.exp(1j * (k0 * j0 + k1 * j1)) / math.sqrt(NA1)
            nd = math.sqrt(abs(d0) ** 2 + abs(d1) ** 2)
            pols = [np.array([1.0, 0.0]), np.array([0.0, 1.0])] if nd == 0.0 else \
                [np.conj(c) / nd, np.array([d0, d1]) / nd]
            for u in pols:
                modes.append((lam, u, M @ u, ph))
    real = sorted([m for m in modes if m[0] > 0], key=lambda m: -m[0])
    evan = sorted([m for m in modes if m[0] <= 0], key=lambda m: -m[0])
    theta = np.zeros(2 * N, np.complex128)
    Xi = np.zeros((2 * N, 2 * N), np.complex128)
    for col, (lam, u, Mu, ph) in enumerate(real + evan):
        s = np.sqrt(complex(lam, 0.0))
        H = np.concatenate([u[0] * ph, u[1] * ph])
        E = np.concatenate([Mu[0] * ph, Mu[1] * ph]) / s
        t = 2.0 * np.arcsin(0.5 * s)
        theta[col], theta[col + N] = t, -t
        Xi[:N, col] = np.exp(-0.5j * t) * H
        Xi[N:, col] = E
        Xi[:N, col + N] = np.exp(0.5j * t) * H
        Xi[N:, col + N] = -E
    nr = len(real)
    for col in range(N):
        f, b = Xi[:, col], Xi[:, col + N]
        if col < nr:
            for v in (f, b):
                z = np.vdot(v[:N], v[N:]) + np.vdot(v[N:], v[:N])
                v *= 1.0 / math.sqrt(abs(z.real))
        else:
            z = np.sqrt(np.vdot(b[:N], f[N:]) + np.vdot(b[N:], f[:N]))
            z = np.conj(z) / (z.real ** 2 + z.imag ** 2)
            f *= z
            b *= np.conj(z)
    return theta, Xi, nr


def grating_layers(L0, L1, nlayers, eps_port=2.085, eps_grating=(2.085, 12.11), fill=0.4, seed=0):
    """Media of nlayers z layers (6, L0*L1) each for the layer-transfer S
    matrix: uniform ports (the first and last layer, matching
    plane_wave_basis) around a seeded two-material pattern (a random
    rectangle of the second material covering about `fill` of each inner
    layer).  Unit cells, mu = 1."""
    rng = np.random.default_rng(seed)
    n = L0 * L1
    j0 = np.tile(np.arange(L0), L1)
    j1 = np.repeat(np.arange(L1), L0)
    out = []
    for z in range(nlayers):
        eps = np.full(n, eps_port, np.complex128)
        if 0 < z < nlayers - 1:
            w0 = max(1, int(round(L0 * math.sqrt(fill))))
            w1 = max(1, int(round(L1 * math.sqrt(fill))))
            a0, a1 = rng.integers(0, L0), rng.integers(0, L1)
            inside = (((j0 - a0) % L0) < w0) & (((j1 - a1) % L1) < w1)
            eps = np.where(inside, eps_grating[1], eps_grating[0]).astype(np.complex128)
        one = np.ones(n, np.complex128)
        out.append(np.stack([one, one, eps, eps, eps, one]))
    return np.array(out)
