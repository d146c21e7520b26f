"""Axis rotation and mirror images of a padded MHD state, for the symmetry
pins of the 3D-only routines.

Arrays are (z, y, x) with two ghost layers.  The rotation maps the old x axis
onto the new y axis, y onto z and z onto x, so an x sweep of a state is a y
sweep of its rotated image; vector components move with their axes and the
face-centred field moves with its faces.  The mirror reverses x: cell i goes
to N + 1 - i and x-face i - 1/2 to face N + 3/2 - i; v_x changes sign, and of
the field only B_x does (a pseudovector mirrors as (Bx, -By, -Bz), and ideal
MHD is symmetric under B -> -B).
"""
import numpy as np

from code_tohoku_gb300 import problems

# EVOLVE's sweep orders (:611-634) and the order that is their rotated image
ROT_ORDER = {1: 2, 2: 3, 3: 1, 4: 5, 5: 6, 6: 4}


def rot(a):
    return np.ascontiguousarray(np.transpose(a, (1, 2, 0)))


def rot_state(st, U=None, sp=None):
    U = st.U if U is None else U
    sp = st.species if sp is None else sp
    out = st.copy()
    src = {0: 0, 4: 4, 1: 3, 2: 1, 3: 2, 5: 7, 6: 5, 7: 6}
    for q in range(8):
        out.U[q] = rot(U[src[q]])
        out.species[q] = rot(sp[q])
    return out


def rot_bcc(b):
    return np.stack([rot(b[2]), rot(b[0]), rot(b[1])])


def _mir_cell(a):
    return np.ascontiguousarray(a[..., ::-1])


def _mir_face(a):
    out = np.empty_like(a)
    out[..., 1:] = a[..., :0:-1]
    out[..., 0] = a[..., -1]
    return out


def mirror_state(st, U=None, sp=None):
    U = st.U if U is None else U
    sp = st.species if sp is None else sp
    out = st.copy()
    for q in range(8):
        if q == 5:
            out.U[q] = -_mir_face(U[q])
        elif q == 1:
            out.U[q] = -_mir_cell(U[q])
        else:
            out.U[q] = _mir_cell(U[q])
        out.species[q] = _mir_cell(sp[q])
    return out


def random_state(n=12, seed=1, mach=1.5, cooling=False):
    """A periodic cube with smooth random rho, p (a few low modes), the
    solenoidal turbulence velocity and a divergence-free face field (curl of
    a random edge vector potential plus a uniform part, no axis special)."""
    st = problems.turbulence(n, mach=mach, kmax=3)
    rng = np.random.default_rng(seed)
    c = (slice(2, -2),) * 3
    k = np.arange(n)

    def smooth():
        f = np.zeros((n, n, n))
        for _ in range(4):
            a, b, cc = rng.integers(0, 3, 3)
            ph = rng.uniform(0, 2 * np.pi, 3)
            f += (rng.normal() * np.cos(2 * np.pi * a * k[:, None, None] / n + ph[0])
                  * np.cos(2 * np.pi * b * k[None, :, None] / n + ph[1])
                  * np.cos(2 * np.pi * cc * k[None, None, :] / n + ph[2]))
        return f

    st.U[0][c] = np.exp(0.3 * smooth())
    st.U[4][c] = 0.6 * np.exp(0.3 * smooth())
    ax, ay, az = (0.3 * smooth() for _ in range(3))
    d = 1.0 / n

    def fwd(f, axis):
        return (np.roll(f, -1, axis=axis) - f) / d
    st.U[5][c] = fwd(az, 1) - fwd(ay, 0) + 0.4
    st.U[6][c] = fwd(ax, 0) - fwd(az, 2) - 0.3
    st.U[7][c] = fwd(ay, 2) - fwd(ax, 1) + 0.2
    problems._fill_ghosts_periodic(st.U)
    if cooling:
        # KI cooling and conduction on (warm gas: T ~ 6000 K at n ~ 1)
        st.params = st.params.replace(ifthrm=2)
        st.U[0] *= 1.27
        st.species[0][...] = st.U[0] / 1.27
        st.U[4] *= 8.63359 * 6.0 / 0.6
    return st
