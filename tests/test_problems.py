"""The synthetic workloads follow their recipes: the reference's ran0 (the
Park-Miller minimal standard; GenDen/IGEN1.f90:169-180, whose MASK XORs are
commented out), the GenDen spectrum fields and the problem set-ups."""
import math

import numpy as np

from code_tohoku_gb300 import problems


def test_ran0_park_miller_known_answer():
    # Park & Miller (1988): from z_1 = 1 the minimal standard gives
    # z_10001 = 1043618065
    vals, idum = problems.ran0_stream(1, 10000)
    assert idum == 1043618065
    assert vals[-1] == idum * 2.0 ** -31


def test_ran0_equals_direct_modular_product():
    for seed in (1, 12345, 2147483646):
        vals, idum = problems.ran0_stream(seed, 257)
        x = seed
        for q in range(257):
            x = 16807 * x % 2147483647
            assert vals[q] == x * 2.0 ** -31
        assert idum == x


def test_solenoidal_velocity_is_divergence_free_at_its_rms():
    n = (12, 10, 16)
    v = problems.solenoidal_velocity(n, vrms=3.0, kmin=1.0, kmax=3.0, idum=7)
    assert v.shape == (3,) + n
    assert math.isclose(np.sqrt(np.mean(np.sum(v * v, axis=0))), 3.0, rel_tol=1e-12)
    # spectral divergence: k . V(k) = 0 for every mode
    V = [np.fft.fftn(v[c]) for c in range(3)]
    kz = np.fft.fftfreq(n[0]) * n[0]
    ky = np.fft.fftfreq(n[1]) * n[1]
    kx = np.fft.fftfreq(n[2]) * n[2]
    KZ, KY, KX = np.meshgrid(kz, ky, kx, indexing="ij")
    div = KX * V[0] + KY * V[1] + KZ * V[2]
    scale = max(np.abs(V[c]).max() for c in range(3))
    assert np.abs(div).max() <= 1e-11 * scale


def test_lognormal_density_has_requested_log_rms():
    n = (16, 16, 16)
    rho = problems.lognormal_density(n, mean=1.27, rms=0.1, kmax=4.0, idum=1)
    lg = np.log(rho / 1.27)
    assert math.isclose(np.sqrt(np.mean(lg * lg)), 0.1, rel_tol=1e-12)
    assert np.all(rho > 0)


def test_uniform_axis_matches_initia():
    x, dx = problems.uniform_axis(8, 20.0)
    assert x.shape == dx.shape == (12,)
    assert np.all(dx == 2.5)
    assert x[1] == 0.0                  # x(0): the left face of cell 1
    assert math.isclose(x[9], 20.0)     # x(n): the right face of cell n
    assert np.allclose(np.diff(x), dx[1:])


def test_turbulence_state():
    st = problems.turbulence(8, mach=5.0, beta=1.0, kmax=2.0)
    inner = (slice(2, -2),) * 3
    g = 5.0 / 3.0
    assert np.all(st.U[0] == 1.0) and np.all(st.U[4] == 1.0 / g)
    v2 = sum(st.U[1 + c][inner] ** 2 for c in range(3))
    assert math.isclose(math.sqrt(np.mean(v2)), 5.0, rel_tol=1e-12)   # rms Mach, sound speed 1
    assert np.all(st.U[5] == math.sqrt(2.0 / g))                        # beta = 2 p / B^2 = 1
    # periodic ghosts: every ghost layer is the image of the opposite interior
    for q in range(8):
        a = st.U[q]
        assert np.array_equal(a[:, :, 0:2], a[:, :, 8:10]) and np.array_equal(a[:, :, 10:12], a[:, :, 2:4])
        assert np.array_equal(a[:, 0:2, :], a[:, 8:10, :]) and np.array_equal(a[0:2], a[8:10])


def test_colliding_flows_state():
    """The benchmark workload: 3 uG at 45 deg in x-y, converging +-20 km/s
    flows, free x and periodic y, z boundaries, T0 = 6000 K, lognormal
    density with a 10 % log rms, WNM species proportional to rho."""
    st = problems.colliding_flows(16)
    p = st.params
    assert p.bc == (1, 1, 3, 3, 3, 3) and p.ifthrm == 2 and p.dissip == 1
    inner = (slice(2, -2),) * 3
    bx, by = st.U[5], st.U[6]
    assert np.allclose(np.hypot(bx, by), 3.0 / 0.448, rtol=1e-15)
    assert np.allclose(bx, by, rtol=1e-15) and np.all(st.U[7] == 0.0)
    lg = np.log(st.U[0][inner] / problems.MU)
    assert math.isclose(np.sqrt(np.mean(lg * lg)), 0.1, rel_tol=1e-12)
    vx = st.U[1][inner][0, 0]
    assert vx[0] > 0.9 * 20.0 / 0.9778 and vx[-1] < -0.9 * 20.0 / 0.9778   # converging at the mid-plane
    # evaluated at the right faces x(i) (:438): antisymmetric about x(n/2) = L/2
    # over cells 1..n-1, zero at cell n/2
    assert np.allclose(vx[:-1], -vx[:-1][::-1], atol=1e-12) and vx[len(vx) // 2 - 1] == 0.0
    # free x sides: both ghost columns copy the first / last interior cell
    for g in (0, 1):
        assert np.array_equal(st.U[:, :, :, g], st.U[:, :, :, 2])
        assert np.array_equal(st.U[:, :, :, -1 - g], st.U[:, :, :, -3])
    # species in fixed proportion to rho; pressure uniform at the mean T0
    ratio = st.species[:, 2:-2, 2:-2, 2:-2] / st.U[0][inner]
    assert np.allclose(ratio, ratio[:, :1, :1, :1], rtol=1e-14)
    ntot = sum(st.species[s][inner] for s in range(5))
    assert np.all(st.U[4] == st.U[4][2, 2, 2])
    assert math.isclose(st.U[4][2, 2, 2] / (problems.KB * np.mean(ntot)), 6.0, rel_tol=1e-14)
