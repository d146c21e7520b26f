"""The output and restart files of SAVEU / SAVEU2D / INITIA and the deck
reader (include/mhd_io.h, code_tohoku_gb300/fortran_io.py).  Host code only.

* every rank's NNNRRR.dat / 000RRR.dat / 2DNNNRRR.dat has the record layout
  of MCF3DSGincfca3.f90:704-710, :749-757, :776-782 (4-byte markers, 17
  values per cell, species order H p H2 He He+ C CO C+, the +1 overlap
  layer) and holds the right global cells for a block decomposition
* a per-rank restart set reads back into the single-domain state
* the D25.17 formatter reproduces the reference's own KIcool/time.DAT lines
* the deck reader parses the shipped 3DMHD-CfCA/INPUT3D.DAT
"""
import os

import numpy as np
import pytest

from code_tohoku_gb300 import fortran_io as fio

NX, NY, NZ = 8, 6, 4
SLOT = [0, 1, 2, 3, 4, 5, 7, 6]   # file slot -> species of the upload order


def records(path, dtype):
    """Fortran unformatted sequential records of a file, as 1D arrays."""
    raw = open(path, "rb").read()
    out, pos = [], 0
    while pos < len(raw):
        n = int(np.frombuffer(raw, "<i4", 1, pos)[0])
        out.append(np.frombuffer(raw, dtype, n // np.dtype(dtype).itemsize, pos + 4))
        assert int(np.frombuffer(raw, "<i4", 1, pos + 4 + n)[0]) == n
        pos += n + 8
    return out


@pytest.fixture
def state():
    rng = np.random.default_rng(3)
    sh = (NZ + 4, NY + 4, NX + 4)
    return rng.normal(size=(8,) + sh), rng.random((8,) + sh), rng.random((3,) + sh), rng.random(sh)


def expected_cell(U, sp, phi, gi, gj, gk, b3=None):
    a = (gk + 1, gj + 1, gi + 1)
    v = [U[q][a] for q in range(5)]
    v += [(b3[q][a] if b3 is not None else U[5 + q][a]) for q in range(3)]
    v += [sp[SLOT[s]][a] for s in range(8)]
    v.append(phi[a] if phi is not None else 0.0)
    return np.array(v)


@pytest.mark.parametrize("nsplit", [(1, 1, 1), (2, 3, 2), (4, 1, 1)])
def test_snapshot_and_restart_layout(tmp_path, state, nsplit):
    U, sp, _, phi = state
    fio.write_snapshot(str(tmp_path), 7, U, sp, phi, nsplit)
    fio.write_restart(str(tmp_path), U, sp, phi, nsplit)
    bx, by, bz = NX // nsplit[0], NY // nsplit[1], NZ // nsplit[2]
    nr = nsplit[0] * nsplit[1] * nsplit[2]
    assert sorted(os.listdir(tmp_path)) == sorted([f"007{r:03d}.dat" for r in range(nr)] +
                                                   [f"000{r:03d}.dat" for r in range(nr)])
    for r in range(nr):
        IS, KS = r % nsplit[0], r // (nsplit[0] * nsplit[1])
        JS = r // nsplit[0] - nsplit[1] * KS
        for name, dt in ((f"007{r:03d}.dat", "<f4"), (f"000{r:03d}.dat", "<f8")):
            recs = records(os.path.join(tmp_path, name), dt)
            assert len(recs) == (bz + 1) * (by + 1)
            q = 0
            for k in range(1, bz + 2):
                for j in range(1, by + 2):
                    rec = recs[q].reshape(bx + 1, 17)
                    q += 1
                    for i in (1, bx // 2 + 1, bx + 1):
                        want = expected_cell(U, sp, phi, IS * bx + i, JS * by + j, KS * bz + k)
                        np.testing.assert_array_equal(rec[i - 1], want.astype(dt))


def test_restart_reads_back_per_rank_set(tmp_path, state):
    U, sp, _, phi = state
    fio.write_restart(str(tmp_path), U, sp, phi, (2, 3, 2))
    U2, sp2, phi2 = fio.read_restart(str(tmp_path), U.shape[1:], (2, 3, 2))
    c = (slice(2, NZ + 3), slice(2, NY + 3), slice(2, NX + 3))   # cells 1..n+1
    np.testing.assert_array_equal(U2[(slice(None),) + c], U[(slice(None),) + c])
    np.testing.assert_array_equal(sp2[(slice(None),) + c], sp[(slice(None),) + c])
    np.testing.assert_array_equal(phi2[c], phi[c])
    assert not U2[:, :2].any() and not U2[:, :, :, :2].any()   # ghosts below 1 untouched
    with pytest.raises(ValueError):
        fio.write_restart(str(tmp_path), U, sp, phi, (3, 1, 1))   # 3 does not divide nx = 8


def test_plane_holds_cell_centred_b(tmp_path, state):
    U, sp, bcc, phi = state
    fio.write_plane(str(tmp_path), 12, U, bcc, sp, None, (2, 1, 2))
    for r in range(4):
        IS, KS = r % 2, r // 2
        recs = records(os.path.join(tmp_path, f"2D012{r:03d}.dat"), "<f4")
        assert len(recs) == NY
        for j in (1, NY):
            rec = recs[j - 1].reshape(NX // 2, 17)
            want = expected_cell(U, sp, None, IS * 4 + 1, j, KS * 2 + 1, b3=bcc)
            np.testing.assert_array_equal(rec[0], want.astype("<f4"))


def test_d25_17_reproduces_reference_time_dat(golden_dir):
    lines = [l.rstrip("\n") for l in open(os.path.join(golden_dir, "ki_time_dat.txt")) if l.strip()]
    assert len(lines) >= 50
    for l in lines:
        v = float(l.replace("D", "E"))
        assert fio.format_d25_17(v, with_1p=False) == l


def test_1p_d25_17_and_info_line(tmp_path):
    assert fio.format_d25_17(0.0) == "  0.00000000000000000D+00"
    assert fio.format_d25_17(0.25) == "  2.50000000000000000D-01"
    assert fio.format_d25_17(-1.5e-120) == " -1.50000000000000005-120"   # 18 digits of the double
    v = 0.57026173842631978
    s = fio.format_d25_17(v)
    assert len(s) == 25 and s.endswith("D-01") and float(s.replace("D", "E")) == v
    fio.write_time_dat(str(tmp_path / "time.DAT"), [0.0, 0.25, 0.5])
    assert open(tmp_path / "time.DAT").read().splitlines()[1] == "  2.50000000000000000D-01"
    fio.write_tsave(str(tmp_path / "tsave.DAT"), 0.5, 3)
    assert open(tmp_path / "tsave.DAT").read().splitlines() == ["  5.00000000000000000D-01", "       3"]
    line = fio.info_line(0.25, 5000, 1.234e-3, "FastSpd")
    assert line == "  2.50000000000000000D-01  Step =    5000  dt =  1.234E-03FastSpd"


def test_saveu_sequence(tmp_path, state):
    U, sp, _, phi = state
    times = []
    n = fio.saveu(str(tmp_path), 1, times, 0.0, 0.0, "FastSpd", 0, U, sp, phi, (2, 1, 1),
                  tfinal=100.0, info_path=str(tmp_path / "info001.DAT"))
    n = fio.saveu(str(tmp_path), n, times, 0.25, 1e-3, "Conduct", 5000, U, sp, phi, (2, 1, 1),
                  tfinal=100.0, info_path=str(tmp_path / "info001.DAT"))
    assert n == 3
    names = set(os.listdir(tmp_path))
    assert {"001000.dat", "001001.dat", "002000.dat", "002001.dat", "000000.dat", "000001.dat",
            "time.DAT", "tsave.DAT", "info001.DAT"} <= names
    assert open(tmp_path / "tsave.DAT").read().splitlines() == ["  2.50000000000000000D-01", "       2"]
    info = open(tmp_path / "info001.DAT").read().splitlines()
    assert info[2].endswith("Conduct") and info[3].startswith("Done ! Time =")


def test_reads_shipped_input3d_deck(golden_dir):
    d = fio.read_input3d(os.path.join(golden_dir, "input3d_deck.txt"))
    assert d.shape == (128, 128, 128) and d.box == (20.0, 20.0, 20.0)
    assert d.vinit[0] == (9.778, -9.778) and d.binit[1] == (2.2307, 2.2307)
    assert (d.cfl, d.facdep, d.maxstp, d.nitera, d.tfinal) == (0.49, 1.0, 4, 5000, 100.0)
    assert d.bc == (4, 4, 3, 3, 3, 3)
    assert (d.ifchem, d.ifthrm, d.ifrad, d.ifgrv) == (2, 2, 0, 0)


def test_reservoir_files_round_trip(tmp_path):
    rng = np.random.default_rng(9)
    sh = (NZ + 4, NY + 4, NX + 4)
    dtf = rng.random(sh).astype(np.float32)
    fio.write_reservoir(str(tmp_path), dtf, (2, 3, 1))
    bx, by, bz = NX // 2, NY // 3, NZ
    for r in range(6):
        IS, JS = r % 2, r // 2
        recs = records(os.path.join(tmp_path, f"D{r:03d}.dat"), "<f4")
        assert len(recs) == bz * by
        np.testing.assert_array_equal(recs[0], dtf[2, JS * by + 2, IS * bx + 2: IS * bx + 2 + bx])
    back = fio.read_reservoir(str(tmp_path), sh, (2, 3, 1), ghost_density=1.25)
    c = (slice(2, NZ + 2), slice(2, NY + 2), slice(2, NX + 2))
    np.testing.assert_array_equal(back[c], dtf[c])
    assert (back[:, :, :2] == np.float32(1.25)).all() and (back[:, :, -2:] == np.float32(1.25)).all()
    np.testing.assert_array_equal(back[2:NZ + 2, 0, 2:NX + 2], back[2:NZ + 2, NY, 2:NX + 2])     # y wrap
    np.testing.assert_array_equal(back[NZ + 3, 2:NY + 2, 2:NX + 2], back[3, 2:NY + 2, 2:NX + 2])  # z wrap


def test_io_errors_are_reported(tmp_path, state):
    """A missing restart set and an unwritable output directory come back as
    the I/O error code (-2, OSError here), not as a partial state."""
    U, sp, _, phi = state
    with pytest.raises(OSError):
        fio.read_restart(str(tmp_path / "empty"), U.shape[1:], (1, 1, 1))
    with pytest.raises(OSError):
        fio.write_restart(str(tmp_path / "no" / "such" / "dir"), U, sp, phi, (1, 1, 1))
