"""mhd_timestep_noalloc: the time-step limits for callers that cannot
allocate device memory (their arrays live in a pool they manage, or new
allocations are not allowed where they call from).  The caller owns every
input; the library's only scratch is a fixed device array.  Checked through
the C ABI against mhd_timestep on the same state, twice in a row (the
shared scratch keeps the previous call's contents), and for the size limit.

Named to be collected last: a run that stops at the first failure has
already run every other test."""
import numpy as np
import pytest

from code_tohoku_gb300 import native, problems

pytestmark = pytest.mark.gpu


def _device_arrays(g, st):
    """The handle's state as caller-owned device arrays.  With the chemistry
    on, nde and ndtot are formed the way mhd_upload forms them (INITIA: the
    same sums in the same order), so they equal the handle's right after an
    upload; SHIELD's columns come from the handle."""
    import torch
    U, sp, bcc = g.download()   # the handle's state, Bcc from its CC(4)
    arrays = [("U", U), ("species", sp), ("bcc", bcc), ("dx", st.dx), ("dy", st.dy), ("dz", st.dz)]
    p = st.params
    if getattr(p, "ifchem", 0) == 2:
        arrays += [("nde", sp[1] + sp[4] + sp[6]), ("ndtot", sp[1] + sp[0] + 2.0 * sp[2] + sp[3] + sp[4])]
        if getattr(p, "ifrad", 0) == 2:
            arrays.append(("columns", g.columns()))
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in arrays}
    torch.cuda.synchronize()
    ds = native.DeviceState(*(dev[k].data_ptr() if k in dev else None for k in
                              ("U", "species", "bcc", "dx", "dy", "dz", "nde", "ndtot", "columns")))
    return ds, dev


@pytest.mark.parametrize("make", [lambda: problems.colliding_flows(32),
                                  lambda: problems.turbulence(24, kmax=4)])
def test_matches_handle_timestep_twice(make):
    st = make()
    g = native.Mhd3D(st.params)
    g.upload(st)
    for _ in range(2):
        ref = g.timestep()
        ds, keep = _device_arrays(g, st)
        got1 = native.timestep_noalloc(st.params, ds)
        got2 = native.timestep_noalloc(st.params, ds)
        assert got1 == ref and got2 == ref
        g.step()   # a different state for the second round


@pytest.mark.parametrize("ifrad", [0, 2])
def test_species_cooling_matches_handle_timestep(ifrad):
    """ifchem = 2 (the shipped deck's chemistry): the thermal limit uses the
    species cooling, which reads nde, ndtot and, with ifrad = 2, SHIELD's
    columns.  Two states: the uploaded one and, re-uploaded into a new
    handle, the state after two steps."""
    from test_chem_oracle import chem_state
    st = chem_state(12, seed=8)
    st.params = st.params.replace(ifchem=2, ifrad=ifrad, ifthrm=2)
    for rnd in range(2):
        g = native.Mhd3D(st.params)
        g.upload(st)
        ref = g.timestep()
        ds, keep = _device_arrays(g, st)
        assert native.timestep_noalloc(st.params, ds) == ref
        assert native.timestep_noalloc(st.params, ds) == ref
        if rnd == 0:
            for _ in range(2):
                g.step()
            U, sp, _ = g.download(with_bcc=False)
            st = st.copy()
            st.U[...] = U
            st.species[...] = sp


def test_species_cooling_needs_its_arrays():
    from test_chem_oracle import chem_state
    st = chem_state(12, seed=8)
    st.params = st.params.replace(ifchem=2, ifrad=2, ifthrm=2)
    g = native.Mhd3D(st.params)
    g.upload(st)
    ds, keep = _device_arrays(g, st)
    ds.columns = None
    with pytest.raises(native.MhdError) as e:
        native.timestep_noalloc(st.params, ds)
    assert e.value.code == 1
    ds.nde = None
    with pytest.raises(native.MhdError) as e:
        native.timestep_noalloc(st.params.replace(ifrad=0), ds)
    assert e.value.code == 1


def test_rejects_grids_beyond_the_scratch():
    import torch
    st = problems.turbulence(16, kmax=2)
    g = native.Mhd3D(st.params)
    g.upload(st)
    ds, keep = _device_arrays(g, st)
    big = st.params.replace(nx=512, ny=256, nz=256)
    assert big.nx * big.ny * big.nz > native.NOALLOC_MAX_CELLS
    with pytest.raises(native.MhdError) as e:
        native.timestep_noalloc(big, ds)
    assert e.value.code == 7
    torch.cuda.synchronize()


def test_matches_chosen_form_handle_timestep():
    """The chosen form keeps the CFL minimum in FP64, so an FP32 handle's
    mhd_timestep equals the allocation-free result on its arrays."""
    st = problems.colliding_flows(32)
    g = native.Mhd3D(st.params, precision=native.PREC_FP32)
    g.upload(st)
    for _ in range(2):
        g.step()
    ref = g.timestep()
    ds, keep = _device_arrays(g, st)
    assert native.timestep_noalloc(st.params, ds, precision=native.PREC_FP32) == ref
    assert native.timestep_noalloc(st.params, ds, precision=native.PREC_FP32) == ref
