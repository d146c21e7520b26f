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
    import torch
    U, sp, bcc = g.download()   # the handle's state, Bcc from its CC(4)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
           (("U", U), ("species", sp), ("bcc", bcc), ("dx", st.dx), ("dy", st.dy), ("dz", st.dz))}
    torch.cuda.synchronize()
    ds = native.DeviceState(*(dev[k].data_ptr() for k in ("U", "species", "bcc", "dx", "dy", "dz")))
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
