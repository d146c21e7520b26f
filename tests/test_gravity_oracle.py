"""Self-gravity on the oracle: the potential of grad^2 Phi = 4 pi G rho,
periodic in y and z and isolated in x (GRAVTY, 3DMHD-CfCA/selfG_MPIfull8.f90).

* the reference's own analytic check (3DMHD-CfCA/Phiexa.f90): a uniform
  slab |x - 50| <= 10 pc in a 100 pc box, rho = 2 / (G4pi 90), has
  Phi = G4pi rho (x - 50)^2 / 2 inside and G4pi rho H |x - 50| - G4pi rho H^2 / 2
  outside; the discrete solution has the exact outer slopes and matches the
  shape to the cell-averaging offset G4pi rho dx^2 / 8;
* the solution satisfies the discrete Poisson equation (second-order x
  Laplacian, three-point y and z Laplacians, periodic) in every cell away
  from the x faces to round-off;
* one y Fourier mode of a thin sheet follows the continuous isolated
  solution -G4pi / (2k) integral rho_k exp(-k |x - x'|) dx' to second order,
  which checks the face values of a k != 0 mode (the sheet sits 2.5 pc from
  a face, where the face value is a few per cent of the peak).
"""
import numpy as np

from code_tohoku_gb300 import problems
from oracle.pyoracle import Oracle3D

G4PI = 12.56637 * 1.11142e-4


def state(nx, ny, nz, lx, rho_of_xyz):
    p = problems.MhdParams(nx, ny, nz, bc=(1, 1, 3, 3, 3, 3), ifthrm=0, dissip=0, ifgrv=2)
    st = problems._empty_state(p, lx, lx * ny / nx, lx * nz / nx)
    cx = st.x - 0.5 * st.dx
    cy = st.y - 0.5 * st.dy
    cz = st.z - 0.5 * st.dz
    st.U[0][...] = rho_of_xyz(cx[None, None, :], cy[None, :, None], cz[:, None, None])
    st.U[4][...] = 1.0
    st.species[0][...] = st.U[0] / 1.27 + 1e-20
    return st, cx, cy, cz


def potential(st):
    o = Oracle3D(st.params)
    o.upload(st)
    return o.potential()


def test_uniform_slab_matches_the_analytic_potential():
    rho0, H, xc = 2.0 / G4PI / 90.0, 10.0, 50.0
    st, cx, _, _ = state(80, 4, 4, 100.0, lambda x, y, z: np.where(np.abs(x - xc) <= H, rho0, 0.0) + 0 * y * z)
    phi = potential(st)[2, 2, 2:-2]
    c = cx[2:-2]
    exact = np.where(np.abs(c - xc) <= H, 0.5 * G4PI * rho0 * (c - xc) ** 2,
                     G4PI * rho0 * H * np.abs(c - xc) - 0.5 * G4PI * rho0 * H * H)
    i0 = int(np.argmin(np.abs(c - xc)))
    d = (phi - phi[i0]) - (exact - exact[i0])
    dx = 100.0 / 80
    assert np.abs(d).max() <= 0.5 * G4PI * rho0 * dx * dx
    # outside the slab the slopes are G4pi rho H exactly
    slope = np.diff(phi) / dx
    assert abs(slope[0] + G4PI * rho0 * H) < 1e-10 and abs(slope[-1] - G4PI * rho0 * H) < 1e-10


def test_discrete_poisson_equation_holds_inside():
    rng = np.random.default_rng(4)
    amp = rng.normal(size=6)

    def rho(x, y, z):
        return (1.0 + 0.3 * amp[0] * np.sin(2 * np.pi * y / 12.0 + amp[1]) * np.cos(2 * np.pi * z / 12.0 + amp[2])
                + 0.2 * np.exp(-((x - 9.0) / 3.0) ** 2) * (1 + amp[3] * np.cos(4 * np.pi * y / 12.0)))
    st, _, _, _ = state(24, 8, 16, 18.0, rho)
    phi = potential(st)
    dx, dy, dz = st.dx[2], st.dy[2], st.dz[2]
    c = (slice(2, -2),) * 3
    lap = ((np.roll(phi, -1, 2) - 2 * phi + np.roll(phi, 1, 2)) / dx ** 2
           + (np.roll(phi, -1, 1) - 2 * phi + np.roll(phi, 1, 1)) / dy ** 2
           + (np.roll(phi, -1, 0) - 2 * phi + np.roll(phi, 1, 0)) / dz ** 2)
    src = G4PI * st.U[0]
    inner = (slice(2, -2), slice(2, -2), slice(3, -3))   # x cells 2..n-1: rows without a face
    err = np.abs(lap[inner] - src[inner]).max()
    assert err <= 1e-12 * np.abs(src[c]).max(), err


def test_a_y_mode_of_a_sheet_follows_the_isolated_solution():
    w, xc, lx, nx, ny = 0.5, 2.5, 20.0, 160, 32   # 2.5 pc from the left face: its value matters
    ly = lx * ny / nx                             # uniform cells: the y box is 4 pc

    def rho(x, y, z):
        return np.where(np.abs(x - xc) <= w, np.cos(2 * np.pi * y / ly), 0.0) + 0 * z
    st, cx, cy, _ = state(nx, ny, 4, lx, rho)
    phi = potential(st)[2, 2:-2, 2:-2]          # (y, x) on the first z row
    c = cx[2:-2]
    dy = st.dy[2]
    k = 2.0 / dy * np.sin(np.pi / ny)            # the discrete y wavenumber of mode 1
    # continuous isolated solution of d^2 f/dx^2 - k^2 f = G4pi rho_k(x), rho_k = 1 on |x - xc| <= w
    xs = np.linspace(xc - w, xc + w, 20001)
    wts = np.full_like(xs, xs[1] - xs[0])
    wts[0] *= 0.5
    wts[-1] *= 0.5
    f = np.array([(-G4PI / (2 * k)) * np.sum(wts * np.exp(-k * np.abs(x - xs))) for x in c])
    amp = phi[:, :].T @ np.cos(2 * np.pi * (cy[2:-2]) / ly) / np.sum(np.cos(2 * np.pi * cy[2:-2] / ly) ** 2)
    assert np.abs(amp - f).max() <= 2e-2 * np.abs(f).max(), np.abs(amp - f).max() / np.abs(f).max()
