"""Run parameters, host-side state and the synthetic initial conditions.

`MhdParams` carries what the reference reads from INPUT3D.DAT and hard-codes
in INITIA (3DMHD-CfCA/MCF3DSGincfca3.f90:134-179): grid, CFL, facdep, tfinal,
the six boundary codes, the floors pmin/pmax/rmin, kb, Kcond and the thermal
and DISSIP switches.  `MhdState` holds the arrays in the reference layout:
U(-1:ndx,-1:ndy,-1:ndz,8) and the eight species arrays, stored as numpy
arrays of shape (8, nz+4, ny+4, nx+4) — x is the unit-stride axis exactly as
in the Fortran column-major arrays.

The problem generators reproduce the workloads the step is benchmarked on
(no datasets are involved; every input is generated from a seed):
  * `brio_wu_deck`      1D Brio-Wu shock tube deck for the 1D driver
  * `ki_shock_tube_deck` the KIcool/INPUT.DAT colliding-flow deck (golden run)
  * `turbulence`        decaying supersonic MHD turbulence, periodic cube
  * `colliding_flows`   warm neutral medium colliding flows with KI cooling
  * `wnm_shock_tube`    the reference's default x shock tube (INITIA:202-253)
Random numbers come from the reference's Park-Miller generator `ran0`
(MCF3DSGincfca3.f90:489-500, GenDen/IGEN1.f90:169-180).
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass
from typing import Tuple

import numpy as np

KB = 8.63359          # p = n kb T with T in 1e3 K (MCF3DSGincfca3.f90:11)
KCOND = 1.6384e-2
MU = 1.27

# species slots (order of the reference's REMAP G(:,1..8))
SPECIES = ("ndH", "ndp", "ndH2", "ndHe", "ndHep", "ndC", "ndCp", "ndCO")

# warm-neutral-medium abundances per H nucleus, MCF3DSGincfca3.f90:156-157
WNM = dict(H=0.9219098, p=0.9503446e-2, H2=0.9465513e-8, He=0.9155226e-1,
           Hep=0.5655353e-3, C=0.1565848e-8, CO=0.2202631e-20, Cp=0.1433520e-3)
XC = 1.4e-4


@dataclass
class MhdParams:
    nx: int
    ny: int
    nz: int
    cfl: float = 0.49
    facdep: float = 1.0
    tfinal: float = 1.0e30
    bc: Tuple[int, int, int, int, int, int] = (3, 3, 3, 3, 3, 3)
    pmin: float = 1.829797 * 8.6336          # MCF3DSGincfca3.f90:173
    pmax: float = 1.0e10
    rmin: float = 0.1949628
    kb: float = KB
    kcond: float = KCOND
    ifthrm: int = 2
    dissip: int = 1
    ifchem: int = 0     # 2: chemistry network + species cooling (the shipped deck's); 0: KI cooling
    ifrad: int = 0      # 2: SHIELD column densities (x sides); 0: columns 0 (the shipped deck's)
    ifgrv: int = 0      # 2: self-gravity (periodic y, z; isolated x); 0: off (the shipped deck's)

    def replace(self, **kw):
        return dataclasses.replace(self, **kw)


def ran0_stream(idum: int, n: int):
    """n successive ran0 draws (Park-Miller minimal standard, Schrage form).

    Returns (values, new_idum).  AM is the single-precision 1./IM of the
    Fortran PARAMETER statement, i.e. exactly 2**-31.
    """
    IA, IM, IQ, IR = 16807, 2147483647, 127773, 2836
    out = np.empty(n, dtype=np.float64)
    am = 2.0 ** -31
    for q in range(n):
        k = idum // IQ
        idum = IA * (idum - k * IQ) - IR * k
        if idum < 0:
            idum += IM
        out[q] = am * idum
    return out, idum


@dataclass
class MhdState:
    params: MhdParams
    U: np.ndarray
    species: np.ndarray
    x: np.ndarray
    dx: np.ndarray
    y: np.ndarray
    dy: np.ndarray
    z: np.ndarray
    dz: np.ndarray
    time: float = 0.0

    @property
    def shape(self):
        p = self.params
        return (p.nz + 4, p.ny + 4, p.nx + 4)

    def coords_vector(self):
        return np.concatenate([self.x, self.dx, self.y, self.dy, self.z, self.dz])

    def interior(self, a):
        return a[..., 2:-2, 2:-2, 2:-2]

    def copy(self):
        return dataclasses.replace(self, U=self.U.copy(), species=self.species.copy())


def uniform_axis(n: int, length: float):
    """x(-1..n+2) and dx(-1..n+2) as built in INITIA (:255-298)."""
    dx = np.full(n + 4, length / n)
    x = np.empty(n + 4)
    x[0] = -dx[1]
    for i in range(1, n + 4):
        x[i] = x[i - 1] + dx[i]
    return x, dx


def _empty_state(p: MhdParams, lx: float, ly: float, lz: float) -> MhdState:
    sh = (p.nz + 4, p.ny + 4, p.nx + 4)
    x, dx = uniform_axis(p.nx, lx)
    y, dy = uniform_axis(p.ny, ly)
    z, dz = uniform_axis(p.nz, lz)
    return MhdState(p, np.zeros((8,) + sh), np.zeros((8,) + sh), x, dx, y, dy, z, dz)


def _centres(x):
    return 0.5 * (x[:-1] + x[1:])


def _fourier_field(n: Tuple[int, int, int], modes, coeff):
    """Sum of coeff_k * exp(i 2 pi k.x) over the listed integer modes,
    evaluated at cell centres (i-1/2)/N; real part returned (float64)."""
    nz, ny, nx = n
    F = np.zeros((nz, ny, nx), dtype=np.complex128)
    l, ll, lll = modes
    # centre offset: exp(i 2 pi k (i - 1/2)/N) = exp(i 2 pi k (i-1)/N) exp(-i pi k / N)
    shift = np.exp(-1j * np.pi * (l / nx + ll / ny + lll / nz))
    np.add.at(F, (lll % nz, ll % ny, l % nx), coeff * shift)
    f = np.fft.ifftn(F) * (nx * ny * nz)
    return f.real


def _integer_modes(kmin: float, kmax: float):
    r = int(math.floor(kmax))
    rng = np.arange(-r, r + 1)
    # loop order of GenDen/IGEN1.f90:102-113: l outer, ll, lll inner
    l, ll, lll = np.meshgrid(rng, rng, rng, indexing="ij")
    l, ll, lll = l.ravel(), ll.ravel(), lll.ravel()
    kw = np.sqrt((l * l + ll * ll + lll * lll).astype(np.float64))
    keep = (kw > 0) & (kw >= kmin) & (kw <= kmax)
    return l[keep], ll[keep], lll[keep], kw[keep]


def lognormal_density(n: Tuple[int, int, int], mean: float, rms: float, kmax: float,
                      slope: float = -11.0 / 3.0, idum: int = 1):
    """GenDen/IGEN1.f90:100-131: sum of cos modes with amplitude
    sqrt(k**slope) and ran0 phases, normalised, then mean*exp(a*field) with
    a chosen so the Gaussian field has rms `rms`."""
    l, ll, lll, kw = _integer_modes(1.0, kmax)
    phases, _ = ran0_stream(idum, len(kw))
    amp = np.sqrt(kw ** slope)
    coeff = amp * np.exp(1j * 2.0 * np.pi * phases)
    f = _fourier_field(n, (l, ll, lll), coeff)
    a = rms / np.sqrt(np.mean(f * f))
    return mean * np.exp(a * f)


def solenoidal_velocity(n: Tuple[int, int, int], vrms: float, kmin: float, kmax: float,
                        slope: float = -4.0, idum: int = 1):
    """Gaussian random velocity: per mode three Box-Muller amplitudes
    (ran0 draws) times sqrt(k**slope), random phase, projected onto the plane
    normal to k (divergence-free), summed at cell centres, scaled to vrms."""
    l, ll, lll, kw = _integer_modes(kmin, kmax)
    m = len(kw)
    r, _ = ran0_stream(idum, 8 * m)
    r = r.reshape(m, 8)
    u1 = np.maximum(r[:, 0:3], 1e-300)
    g = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * r[:, 3:6])
    ph = np.exp(1j * 2.0 * np.pi * r[:, 6])
    vk = g * np.sqrt(kw ** slope)[:, None]
    kvec = np.stack([l, ll, lll], axis=1).astype(np.float64)
    vk = vk - kvec * (np.sum(kvec * vk, axis=1) / (kw * kw))[:, None]
    comps = [_fourier_field(n, (l, ll, lll), vk[:, c] * ph) for c in range(3)]
    v = np.stack(comps)
    s = vrms / np.sqrt(np.mean(np.sum(v * v, axis=0)))
    return v * s


def _fill_ghosts_periodic(a):
    """Periodic images for every ghost cell (2 deep) of an (..., z, y, x) array."""
    for ax in (-1, -2, -3):
        n = a.shape[ax] - 4
        sl = [slice(None)] * a.ndim

        def put(dst, src):
            d = list(sl); d[ax] = dst
            s = list(sl); s[ax] = src
            a[tuple(d)] = a[tuple(s)]
        put(slice(0, 2), slice(n, n + 2))
        put(slice(n + 2, n + 4), slice(2, 4))
    return a


def turbulence(n: int = 128, mach: float = 5.0, beta: float = 1.0, gamma: float = 5.0 / 3.0,
               kmax: float = 8.0, idum: int = 1, cfl: float = 0.4) -> MhdState:
    """Decaying supersonic MHD turbulence: periodic unit cube, rho=1,
    p=1/gamma (sound speed 1), solenoidal k^-4 velocity on |k|=1..8 at rms
    Mach `mach`, uniform Bx with plasma beta `beta`; no cooling, no DISSIP,
    floors lowered so the dimensionless state is never clamped."""
    p = MhdParams(n, n, n, cfl=cfl, bc=(3, 3, 3, 3, 3, 3), pmin=1e-20, pmax=1e20, rmin=1e-20,
                  ifthrm=0, dissip=0)
    st = _empty_state(p, 1.0, 1.0, 1.0)
    pres = 1.0 / gamma
    v = solenoidal_velocity((n, n, n), mach, 1.0, kmax, idum=idum)
    inner = (slice(2, -2),) * 3
    st.U[0][...] = 1.0
    st.U[4][...] = pres
    for c in range(3):
        st.U[1 + c][inner] = v[c]
    st.U[5][...] = math.sqrt(2.0 * pres / beta)
    # hydrogen only: gamma = 5/3 from the species formula (H2 = 0)
    st.species[0][...] = 1.0
    _fill_ghosts_periodic(st.U)
    return st


def colliding_flows(n: int = 256, box: float = 20.0, n0: float = 1.0, T0: float = 6.0,
                    vflow: float = 20.0 / 0.9778, bmag: float = 3.0 / 0.448, angle_deg: float = 45.0,
                    rms: float = 0.1, pert_scale: float = None, idum: int = 1) -> MhdState:
    """Warm-neutral-medium colliding flows with KI cooling: cube of `box` pc,
    n0 [cm^-3] (rho = 1.27 n0), T0 in 1e3 K, lognormal rho with rms 0.1 and
    k^-11/3 (GenDen recipe, kmax = N/4 or box/pert_scale), converging
    vx = -v tanh((x - L/2)/2) (MCF3DSGincfca3.f90:438), |B| in code units at
    `angle_deg` to x in the x-y plane, free x boundaries, periodic y and z,
    species proportional to rho with the WNM ratios (BBRV_cm, :182-189)."""
    p = MhdParams(n, n, n, cfl=0.49, bc=(1, 1, 3, 3, 3, 3), ifthrm=2, dissip=1)
    st = _empty_state(p, box, box, box)
    kmax = n / 4.0 if pert_scale is None else box / pert_scale
    rho = lognormal_density((n, n, n), MU * n0, rms, kmax, idum=idum)
    inner = (slice(2, -2),) * 3
    st.U[0][inner] = rho
    xi = st.x[2:-2]            # x(i), i = 1..N (right edges), as in :438
    vx = -vflow * np.tanh(0.5 * (xi - 0.5 * box))
    st.U[1][inner] = vx[None, None, :]
    th = math.radians(angle_deg)
    st.U[5][...] = bmag * math.cos(th)
    st.U[6][...] = bmag * math.sin(th)
    # species per unit mass density (BBRV_cm, MCF3DSGincfca3.f90:182-189)
    w = WNM
    cm = np.array([0.91 / MU, 0.91 * w["p"] / w["H"] / MU, 0.91 * w["H2"] / w["H"] / MU,
                   0.09 / MU, 0.09 * w["Hep"] / w["He"] / MU,
                   XC * w["C"] / w["Cp"] / MU, XC / MU, XC * w["CO"] / w["Cp"] / MU])
    # order of our slots: H, p, H2, He, Hep, C, Cp, CO
    _fill_ghosts_periodic(st.U)
    # free x boundary: ghost columns copy the first/last interior cell
    for g in (0, 1):
        st.U[:, :, :, g] = st.U[:, :, :, 2]
        st.U[:, :, :, -1 - g] = st.U[:, :, :, -3]
    for s in range(8):
        st.species[s] = cm[s] * st.U[0]
    ntot = st.species[0] + st.species[1] + st.species[2] + st.species[3] + st.species[4]
    st.U[4][...] = np.mean(ntot[inner]) * KB * T0
    return st


def wnm_shock_tube(n: int = 64, box: float = 20.0, vflow: float = 9.778, by=(2.2307, 2.2307),
                   bc=(4, 4, 3, 3, 3, 3), ifthrm: int = 2, dissip: int = 1) -> MhdState:
    """The reference's default x shock tube (MCF3DSGincfca3.f90:202-253) with
    the shipped deck values (3DMHD-CfCA/INPUT3D.DAT): WNM (dinit1, p/kB = 8810
    K cm^-3) moving at +vflow for i <= n/2 and -vflow beyond, By = binity1 /
    binity2 on the two sides.  bc selects the boundary codes; the shipped deck
    uses the inflow code 4 in x, whose data are `shock_tube_inflow(...)`."""
    p = MhdParams(n, n, n, cfl=0.49, bc=tuple(bc), ifthrm=ifthrm, dissip=dissip)
    st = _empty_state(p, box, box, box)
    w = WNM
    d = w["H"] + w["p"] + 2.0 * w["H2"] + 4.0 * w["He"] + 4.0 * w["Hep"]
    pinit = 8.810807e3 * KB * 1.0e-3
    left = (np.arange(n + 4) - 1) <= n // 2
    st.U[0][...] = d
    st.U[1][...] = np.where(left, vflow, -vflow)[None, None, :]
    st.U[4][...] = pinit
    st.U[6][...] = np.where(left, by[0], by[1])[None, None, :]
    for s, key in enumerate(("H", "p", "H2", "He", "Hep", "C", "Cp", "CO")):
        st.species[s][...] = w[key]
    return st


def shock_tube_inflow(vflow: float = 9.778, by=(2.2307, 2.2307)) -> Tuple["Inflow", float]:
    """BC=4 data of the default shock tube: the inflow values of INITIA and
    the uniform DTF reservoir dinit1 (the shipped code skips the DTF file
    read, :402-404)."""
    w = WNM
    dinit = w["H"] + w["p"] + 2.0 * w["H2"] + 4.0 * w["He"] + 4.0 * w["Hep"]
    return reference_inflow((vflow, 0.0, 0.0), (0.0, by[0], 0.0), (0.0, by[1], 0.0)), dinit


@dataclass
class Inflow:
    """BC=4 inflow data (BBRV, BBRV_cm of INITIA :182-200): the values a ghost
    cell on an inflow side of x receives.  Side 0 is x = 0, side 1 the far
    end.  `species` is the number density per unit mass density in the
    upload order (H, p, H2, He, He+, C, C+, CO)."""
    rho_ref: float
    v: Tuple[Tuple[float, float, float], Tuple[float, float, float]]
    p: Tuple[float, float]
    b: Tuple[Tuple[float, float, float], Tuple[float, float, float]]
    species: Tuple[float, ...]

    def vector(self):
        return np.array([self.rho_ref, *self.v[0], *self.v[1], *self.p, *self.b[0], *self.b[1],
                         *self.species], dtype=np.float64)


def reference_inflow(vinit, binit1, binit2, pinit=8.810807e3 * KB * 1.0e-3) -> Inflow:
    """INITIA's inflow values (:182-200) for the deck's vinit = (vx, vy, vz) of
    side 1 and binit1/binit2 of the two sides: species fractions of the WNM
    scaled to unit mass density, reference density dBC, the right side's
    inflow velocity -vx."""
    w = WNM
    cm_H, cm_p = 0.91 / 1.27, 0.91 * w["p"] / w["H"] / 1.27
    cm_H2, cm_He = 0.91 * w["H2"] / w["H"] / 1.27, 0.09 / 1.27
    cm_Hep = 0.09 * w["Hep"] / w["He"] / 1.27
    cm_Cp = XC / 1.27
    cm_C = XC * w["C"] / w["Cp"] / 1.27
    cm_CO = XC * w["CO"] / w["Cp"] / 1.27
    dbc = 1.0 * cm_H + 1.0 * cm_p + 2.0 * cm_H2 + 4.0 * cm_He + 4.0 * cm_Hep
    vx, vy, vz = vinit
    return Inflow(rho_ref=dbc, v=((vx, vy, vz), (-vx, vy, vz)), p=(pinit, pinit),
                  b=(tuple(binit1), tuple(binit2)),
                  species=(cm_H, cm_p, cm_H2, cm_He, cm_Hep, cm_C, cm_Cp, cm_CO))


def _deck_vector(Np1x, Np2x, ql1x, ql2x, d, vx, vy, vz, pp, bx, by, bz, spec, cfl, facdep,
                 tfinal, bc, ifthrm, brio_wu, p_override):
    v = [Np1x, Np2x, ql1x, ql2x, *d, *vx, *vy, *vz, *pp, *bx, *by, *bz]
    for pair in spec:
        v += list(pair)
    v += [cfl, facdep, 0, tfinal, bc[0], bc[1], ifthrm, brio_wu, p_override]
    return np.array(v, dtype=np.float64)


def ki_shock_tube_deck():
    """KIcool/INPUT.DAT with the pressure override of KIcool/1DMHDwCC3.f90:82-83."""
    spec = [(1.0, 1.0)] + [(0.0, 0.0)] * 7
    return _deck_vector(512, 512, 10.0, 10.0, (1.0, 1.0), (48.89, -48.89), (0, 0), (0, 0),
                        (1.0, 0.1), (1.57734, 1.57734), (1.57734, 1.57734), (0, 0), spec,
                        0.49, 1.0, 40.0, (1, 1), 2, 0, 8.810807e3 * KB * 1.0e-3)


def brio_wu_deck(ncell: int = 800, tfinal: float = 0.1, cfl: float = 0.5):
    """Brio-Wu on [0,1] (1DMHDmany/1DMHDwCC3bw.f90 with INPUT/INPUT.DAT values):
    (rho,p,By) = (1,1,1) | (0.125,0.1,-1), Bx = 0.75, gamma = 2 in the sound
    speed and CFL, free boundaries, no source."""
    h = ncell // 2
    spec = [(1.0, 0.125)] + [(0.0, 0.0)] * 7
    return _deck_vector(h, h, 0.5, 0.5, (1.0, 0.125), (0, 0), (0, 0), (0, 0), (1.0, 0.1),
                        (0.75, 0.75), (1.0, -1.0), (0, 0), spec, cfl, 1.0, tfinal, (1, 1), 0, 1, -1.0)
