"""The oracle's chemistry network (ifchem = 2: SOURCE's CHEM branch and the
species cooling of Fcool, 3DMHD-CfCA/MCF3DSGincfca3.f90:2576-2776,
:2825-2880, RATES :3037-3131) checked through properties the network has by
construction: every reaction moves nuclei between species of one element, so
the H, He and C nuclei of each cell are conserved by a source step wherever
no density floor acts (the floors ndHmin = 0.91 rmin, ndHemin = 0.09 rmin
and 1e-20 for the rest, :178 and :2759-2766, add nuclei); densities stay
positive; and the network does something (a hot cell ionises, a cold dense
cell forms H2)."""
import numpy as np

from code_tohoku_gb300 import problems
from oracle.pyoracle import Oracle3D

C = (slice(2, -2),) * 3


def nuclei(sp):
    """H, He, C nuclei per cell (species order H, p, H2, He, He+, C, C+, CO)."""
    return (sp[0] + sp[1] + 2.0 * sp[2], sp[3] + sp[4], sp[5] + sp[6] + sp[7])


def chem_state(n=12, seed=3):
    st = problems.wnm_shock_tube(n, bc=(3, 3, 3, 3, 3, 3))
    st.params = st.params.replace(ifchem=2)
    rng = np.random.default_rng(seed)
    # a spread of densities (x1/30 .. x30) and temperatures around the WNM
    f = np.exp(rng.uniform(-3.4, 3.4, size=st.U[0].shape))
    st.U[0] *= f
    for s in range(8):
        st.species[s] *= f
    st.U[4] *= np.exp(rng.uniform(-2.0, 4.0, size=st.U[0].shape))
    return st


def floored(sp, rmin):
    """Cells where the H or He floor may have acted (the 1e-20 floors add
    at most a few 1e-20 and are covered by the absolute tolerance)."""
    return (sp[0] <= 0.91 * rmin * (1 + 1e-9)) | (sp[3] <= 0.09 * rmin * (1 + 1e-9))


def test_chem_source_conserves_nuclei():
    st = chem_state()
    o = Oracle3D(st.params)
    o.upload(st)
    _, sp0, _ = o.download()
    o.source(0.05)
    U1, sp1, _ = o.download()
    free = ~floored(sp1, st.params.rmin)[C]
    assert free.mean() > 0.5
    for a, b in zip(nuclei(sp0), nuclei(sp1)):
        np.testing.assert_allclose(b[C][free], a[C][free], rtol=1e-11, atol=1e-19)
    # the floors only add nuclei
    assert np.all(nuclei(sp1)[0][C] >= nuclei(sp0)[0][C] * (1 - 1e-11))
    assert np.all(sp1[:, C[0], C[1], C[2]] >= 0.0)
    assert np.all(np.isfinite(U1[:, C[0], C[1], C[2]]))
    # the network changed the composition
    assert np.max(np.abs(sp1[1][C] - sp0[1][C]) / sp0[1][C]) > 1e-3


def test_chem_hot_cells_ionise_cold_dense_cells_form_h2():
    st = chem_state(seed=4)
    o = Oracle3D(st.params)
    o.upload(st)
    _, sp0, _ = o.download()
    ntot = sp0[0] + sp0[1] + sp0[2] + sp0[3] + sp0[4]
    T = st.U[4] / st.params.kb / ntot
    for _ in range(20):
        o.source(0.05)
    _, sp1, _ = o.download()
    hot = (T > 8.0)[C]            # T in 1e3 K
    dh = (sp1[1] / sp0[1])[C]
    assert np.median(dh[hot]) > 1.0
    cold = ((T < 0.3) & (st.U[0] > 10.0))[C]
    if cold.any():
        assert np.median((sp1[2] / sp0[2])[C][cold]) > 1.0


def test_chem_steps_stay_finite():
    st = problems.wnm_shock_tube(16, bc=(3, 3, 3, 3, 3, 3))
    st.params = st.params.replace(ifchem=2)
    o = Oracle3D(st.params)
    o.upload(st)
    _, sp0, _ = o.download()
    for _ in range(10):
        o.step()
    U, sp, _ = o.download()
    assert np.all(np.isfinite(U[:, C[0], C[1], C[2]]))
    assert np.all(sp[:, C[0], C[1], C[2]] > 0.0)
    # periodic box: the nuclei totals are conserved by advection and network
    for a, b in zip(nuclei(sp0), nuclei(sp)):
        np.testing.assert_allclose(b[C].sum(), a[C].sum(), rtol=1e-10)


def shield_state(n=12, seed=5):
    st = chem_state(n, seed)
    st.params = st.params.replace(ifrad=2)
    return st


def column_totals(o, st):
    """Σ dx ndtot along x of every (j, k) line, from the species of the state
    the oracle holds (ndtot of INITIA, :473)."""
    _, sp, _ = o.download()
    ndtot = sp[1] + sp[0] + 2.0 * sp[2] + sp[3] + sp[4]
    return (ndtot[C] * st.dx[2]).sum(axis=2)


def test_shield_columns_split_the_line_total():
    """SHIELD (:2924-3036): the column from the left plus the column from the
    right of every cell is the whole line's column Σ dx ndtot."""
    st = shield_state()
    o = Oracle3D(st.params)
    o.upload(st)
    cols = o.columns()
    tot = column_totals(o, st)
    np.testing.assert_allclose((cols[0] + cols[1])[C], np.repeat(tot[:, :, None], st.params.nx, axis=2),
                               rtol=1e-12)
    # the left columns grow along x, the right ones shrink
    assert np.all(np.diff(cols[0][C], axis=2) > 0) and np.all(np.diff(cols[1][C], axis=2) < 0)
    # H2, C and CO columns likewise split their line totals
    _, sp, _ = o.download()
    for q, s in ((1, 2), (2, 5), (3, 7)):
        line = (sp[s][C] * st.dx[2]).sum(axis=2)
        np.testing.assert_allclose((cols[2 * q] + cols[2 * q + 1])[C],
                                   np.repeat(line[:, :, None], st.params.nx, axis=2), rtol=1e-12)


def test_shield_changes_the_microphysics():
    """With columns the species cooling and the rates see shielding: the
    same source step gives a different state than with ifrad = 0."""
    st = shield_state()
    outs = []
    for ifrad in (0, 2):
        o = Oracle3D(st.params.replace(ifrad=ifrad))
        o.upload(st)
        o.source(0.05)
        outs.append(o.download())
    assert not np.array_equal(outs[0][0][4], outs[1][0][4])
    assert not np.array_equal(outs[0][1][2], outs[1][1][2])
