"""Self-gravity on the GPU (ifgrv = 2) against the oracle.

The GPU transforms y and z with radix-4 FFTs in shared memory (two real
z rows per complex y transform, then the half spectrum), the oracle with
plain DFTs of every mode, and the GPU's x solve reads tabulated Green's
weights and elimination coefficients, so the potentials agree to round-off,
not bit for bit.  Also the
analytic slab of the reference's Phiexa.f90 on the GPU, whole steps of both
forms with gravity on, and mhd_step_host with gravity equal to upload +
step + download bit for bit."""
import numpy as np
import pytest

from code_tohoku_gb300 import native, problems
from oracle.pyoracle import Oracle3D
from test_gravity_oracle import G4PI, state

pytestmark = pytest.mark.gpu
C = (slice(2, -2),) * 3


def blob_state(nx, ny, nz, seed=1):
    rng = np.random.default_rng(seed)
    a = rng.normal(size=4)
    lx = 20.0

    def rho(x, y, z):
        ly, lz = lx * ny / nx, lx * nz / nx
        return (1.27 * (1.0 + 0.2 * np.sin(2 * np.pi * y / ly + a[0]) * np.cos(2 * np.pi * z / lz + a[1]))
                * (1.0 + 4.0 * np.exp(-((x - 0.4 * lx) / 2.0) ** 2 - ((y - 0.5 * ly) / 2.5) ** 2)))
    st, _, _, _ = state(nx, ny, nz, lx, rho)
    st.U[4][...] = 51.8 * st.U[0] / 1.27
    st.U[1][...] = 0.5 * a[2]
    st.U[5][...] = 2.0
    st.U[6][...] = 1.0
    st.species[0][...] = st.U[0] / 1.27
    problems._fill_ghosts_periodic(st.U)
    for g in (0, 1):
        st.U[:, :, :, g] = st.U[:, :, :, 2]
        st.U[:, :, :, -1 - g] = st.U[:, :, :, -3]
    return st


@pytest.mark.parametrize("shape", [(16, 16, 16), (24, 8, 32), (20, 64, 4), (12, 256, 8), (10, 4, 8), (12, 8, 4)])
def test_potential_matches_the_oracle(shape):
    st = blob_state(*shape)
    g = native.Mhd3D(st.params)
    g.upload(st)
    o = Oracle3D(st.params)
    o.upload(st)
    pg, po = g.potential(), o.potential()
    full = (slice(None),) * 3
    assert np.abs(pg[full] - po[full]).max() <= 1e-12 * np.abs(po).max()


def test_potential_after_a_new_upload_with_other_coordinates():
    """The Green's weights and elimination coefficients are tabulated from
    the grid: a second upload with another box size must rebuild them."""
    st1 = blob_state(16, 16, 16, seed=2)
    g = native.Mhd3D(st1.params)
    g.upload(st1)
    g.potential()
    st2, _, _, _ = state(16, 16, 16, 37.0, lambda x, y, z: 1.0 + 0.5 * np.cos(2 * np.pi * y / 37.0) * np.exp(-((x - 12.0) / 5.0) ** 2) + 0 * z)
    st2.U[4][...] = 51.8 * st2.U[0] / 1.27
    st2.species[0][...] = st2.U[0] / 1.27
    g.upload(st2)
    o = Oracle3D(st2.params)
    o.upload(st2)
    pg, po = g.potential(), o.potential()
    assert np.abs(pg - po).max() <= 1e-12 * np.abs(po).max()


def test_uniform_slab_on_the_gpu():
    rho0, H, xc = 2.0 / G4PI / 90.0, 10.0, 50.0
    st, cx, _, _ = state(80, 4, 4, 100.0, lambda x, y, z: np.where(np.abs(x - xc) <= H, rho0, 0.0) + 0 * y * z)
    g = native.Mhd3D(st.params.replace(rmin=1e-30, pmin=1e-30))
    g.upload(st)
    phi = g.potential()[2, 2, 2:-2]
    c = cx[2:-2]
    exact = np.where(np.abs(c - xc) <= H, 0.5 * G4PI * rho0 * (c - xc) ** 2,
                     G4PI * rho0 * H * np.abs(c - xc) - 0.5 * G4PI * rho0 * H * H)
    i0 = int(np.argmin(np.abs(c - xc)))
    d = (phi - phi[i0]) - (exact - exact[i0])
    assert np.abs(d).max() <= 0.5 * G4PI * rho0 * (100.0 / 80) ** 2


@pytest.mark.parametrize("precision,tol", [(native.PREC_FP64, 1e-10), (native.PREC_FP32, 1e-4)])
def test_steps_with_gravity_match_the_oracle(precision, tol):
    st = blob_state(16, 16, 16, seed=2)
    g = native.Mhd3D(st.params, precision=precision)
    g.upload(st)
    o = Oracle3D(st.params)
    o.upload(st)
    for _ in range(4):
        dt, _ = o.timestep()
        o.advance(dt)
        g.advance(dt)
    Ug, _, _ = g.download()
    Uo, _, _ = o.download()
    for q in (0, 1, 2, 3, 4):
        err = float(np.abs(Ug[q][C] - Uo[q][C]).max() / np.abs(Uo[q][C]).max())
        assert err <= tol, (q, err)
    assert np.abs(g.potential() - o.potential()).max() <= max(tol, 1e-12) * np.abs(o.potential()).max()


def test_step_host_with_gravity_equals_upload_step_download():
    st = blob_state(16, 16, 16, seed=3)
    a = native.Mhd3D(st.params)
    a.upload(st)
    b = native.Mhd3D(st.params)
    b.upload(st)
    U0 = np.ascontiguousarray(st.U)
    S0 = np.ascontiguousarray(st.species)
    Uout, Sout = np.empty_like(U0), np.empty_like(S0)
    ra = a.step_host(U0, S0, Uout, Sout)
    rb = b.step()
    assert ra == rb
    Ub, Sb, _ = b.download(with_bcc=False)
    assert np.array_equal(Uout, Ub) and np.array_equal(Sout, Sb)
    assert np.array_equal(a.potential(), b.potential())


def test_gravity_entry_point_parts_equal_advance():
    """A driver calling the step's parts one by one, with mhd_gravity where
    EVOLVE calls GRAVTY (:607, :653), gets mhd_advance's result bit for bit."""
    st = blob_state(16, 16, 16, seed=4)
    a = native.Mhd3D(st.params)
    a.upload(st)
    b = native.Mhd3D(st.params)
    b.upload(st)
    for k in range(3):
        dt, _ = a.timestep()
        a.advance(dt)
        b.set_time(b.time, k + 1)
        b.gravity(dt, 3)
        b.source(0.5 * dt)
        for d in ((0, 1, 2), (1, 2, 0), (2, 0, 1))[k]:
            b.sweep(d, dt)
        b.ct(dt)
        b.source(0.5 * dt)
        b.gravity(dt, 2)
        b.gravity(dt, 3)
        b.set_time(b.time + dt, k + 2)
    Ua, Sa, _ = a.download(with_bcc=False)
    Ub, Sb, _ = b.download(with_bcc=False)
    assert np.array_equal(Ua, Ub) and np.array_equal(Sa, Sb)
    assert np.array_equal(a.potential(), b.potential())
