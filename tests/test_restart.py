"""RESTART wavefunction files (gbcp_restart_write / gbcp_restart_read, host code
of the C ABI) against the layout restated in oracle/restart_oracle.py: files
written by the library are read by the oracle and the reverse, sequential and
STREAM files, every compression type, plane-wave and state-count changes, the
wavefunction velocities, the occupation and eigenvalue sections behind skipped
ones, and malformed files.
No GPU is involved."""
import struct

import numpy as np
import pytest

from oracle import restart_oracle as RO


@pytest.fixture(scope="module")
def lib():
    from cpmd_gb300 import build as B
    B.build()
    from cpmd_gb300 import _lib
    return _lib.load()


def states(ngw, n, seed):
    rng = np.random.default_rng(seed)
    c = (rng.standard_normal((ngw, n)) + 1j * rng.standard_normal((ngw, n))) * 0.1
    c[0, 0] = 3.0  # one dominant coefficient: every component lies below the izamax scale
    return np.asfortranarray(c)


def cell(seed=7):
    rng = np.random.default_rng(seed)
    na = np.array([3, 2], np.int32)
    tau0 = rng.uniform(0, 10, (5, 3))
    return na, tau0


def test_library_file_read_by_oracle(lib, tmp_path):
    from cpmd_gb300.restart import write_restart
    na, tau0 = cell()
    c = states(211, 9, 1)
    p = tmp_path / "RESTART.1"
    write_restart(p, c, na=na, tau0=tau0, taum=tau0 * 1e-3, ecut=25.0, nel=18, nr=(36, 36, 40), alat=10.26,
                  nhgs=1700, icompr=1)
    d = RO.read(p)
    assert not d["stream"]
    assert d["ibrav"] == 1 and d["indpg"] == 0
    assert np.array_equal(d["celldm"], [10.26, 1.0, 1.0, 0.0, 0.0, 0.0])
    assert np.array_equal(d["na"], na)
    assert np.array_equal(d["tau0"], tau0) and np.array_equal(d["taum"], tau0 * 1e-3) and "taui" not in d
    assert (d["ecut"], d["cdual"], d["nel"], d["nr"]) == (25.0, 4.0, 18, (36, 36, 40))
    assert (d["nstate"], d["nkpts"], d["ngwks"], d["nhgs"]) == (9, 0, 211, 1700)
    assert d["iwfntype"] == 1 and d["icompr"] == 1
    assert d["scale"] == RO.izamax_scale(c)
    assert np.array_equal(d["c0"], c)  # FP64 as is: bit-identical


def test_library_compressed_file_read_by_oracle(lib, tmp_path):
    from cpmd_gb300.restart import read_restart, write_restart
    na, tau0 = cell()
    c = states(128, 5, 2)
    p = tmp_path / "RESTART.2"
    write_restart(p, c, na=na, tau0=tau0, ecut=20.0, nel=10, nr=32, alat=9.0, icompr=2)
    d = RO.read(p)
    mine = read_restart(p)
    assert d["icompr"] == 2 and mine.icompr == 2
    # both decoders agree bit for bit; the reference's decoder drops the last coefficient
    assert np.array_equal(mine.c0, d["c0"])
    assert np.all(d["c0"][-1] == 0)
    err = np.abs(d["c0"][:-1] - c[:-1]).max()
    assert err <= 0.5 * d["scale"] / (2 ** 31 - 1) * 1.0001 * np.sqrt(2)
    # and the words equal the oracle's packing of the same data
    q = tmp_path / "RESTART.2o"
    RO.write(q, c, na=na, tau0=tau0, ecut=20.0, nel=10, nr=32, celldm=[9.0, 1, 1, 0, 0, 0], icompr=2)
    assert p.read_bytes() == q.read_bytes()


@pytest.mark.parametrize("stream", [False, True])
@pytest.mark.parametrize("icompr", [1, 2, 4, 8])
def test_oracle_file_read_by_library(lib, tmp_path, stream, icompr):
    from cpmd_gb300.restart import read_restart
    na, tau0 = cell(3)
    c = states(160, 6, 3 + icompr)  # 2 ngw a multiple of 8: every packing keeps whole words
    p = tmp_path / "RESTART.o"
    RO.write(p, c, na=na, tau0=tau0, taui=tau0 + 1.0, ecut=30.0, nel=12, nr=(40, 40, 48),
             celldm=[11.0, 1.0, 1.2, 0.0, 0.0, 0.0], icompr=icompr, stream=stream, dual=True, nhgs=999)
    ref = RO.read(p)
    d = read_restart(p)
    assert d.icompr == icompr and d.nstate == 6 and d.nstate_file == 6 and d.ngwks == 160
    assert np.array_equal(d.na, na) and np.array_equal(d.tau0, tau0) and d.taum is None
    assert np.array_equal(d.taui, tau0 + 1.0)
    assert np.array_equal(d.celldm, [11.0, 1.0, 1.2, 0.0, 0.0, 0.0])
    assert (d.ecut, d.nel, d.nr, d.dual, d.nhgs) == (30.0, 12, (40, 40, 48), True, 999)
    assert np.array_equal(d.c0, ref["c0"])
    if icompr == 1:
        assert np.array_equal(d.c0, c)
    else:
        nb = 64 // icompr
        assert np.abs(d.c0[:-4] - c[:-4]).max() <= d.scale / (2 ** (nb - 1) - 1)
    for k in (1, 2, 3, 4, 6, 7, 8, 9):
        assert d.has_section(k)
    assert not d.has_section(5)


def test_plane_wave_and_state_changes(lib, tmp_path):
    """rdwfn stores min(ngw, ngwks) rows and zeroes the rest; r_wfnio reads
    min(nstate, file) states."""
    from cpmd_gb300.restart import read_restart, write_restart
    na, tau0 = cell()
    c = states(100, 8, 4)
    p = tmp_path / "RESTART.3"
    write_restart(p, c, na=na, tau0=tau0, ecut=20.0, nel=16, nr=32, alat=10.0)
    big = read_restart(p, ngw=130, nstate=5)
    assert big.c0.shape == (130, 5)
    assert np.array_equal(big.c0[:100], c[:, :5]) and np.all(big.c0[100:] == 0)
    small = read_restart(p, ngw=60)
    assert small.c0.shape == (60, 8) and np.array_equal(small.c0, c[:60])


def test_basis_states_round_trip(lib, tmp_path):
    """States of a basis made in the reference's G order come back row for row."""
    from cpmd_gb300.restart import read_restart, write_restart
    from cpmd_gb300.synth import make_small_cell
    cl = make_small_cell(10.26, 32, 20.0, 12, seed=5)
    b = cl.basis
    p = tmp_path / "RESTART.cell"
    write_restart(p, cl.c0, na=[4], tau0=np.zeros((4, 3)), ecut=b.ecut, nel=24, nr=b.nr, alat=b.alat,
                  nhgs=b.nhg)
    d = read_restart(p, ngw=b.ngw)
    assert d.ngwks == b.ngw and d.nhgs == b.nhg
    assert np.array_equal(d.c0, cl.c0)


def _status(lib, path):
    from cpmd_gb300 import _lib
    import ctypes as C
    r = _lib.Restart()
    return lib.gbcp_restart_read(str(path).encode(), C.byref(r))


def test_malformed_files_are_reported(lib, tmp_path):
    na, tau0 = cell()
    c = states(64, 3, 5)
    good = tmp_path / "RESTART.good"
    RO.write(good, c, na=na, tau0=tau0, ecut=20.0, nel=6, nr=32, celldm=[10, 1, 1, 0, 0, 0])
    data = good.read_bytes()
    assert _status(lib, good) == 0
    assert _status(lib, tmp_path / "missing") == 9
    (tmp_path / "trunc").write_bytes(data[:200])  # inside section 4
    assert _status(lib, tmp_path / "trunc") == 9
    (tmp_path / "trunc9").write_bytes(data[:len(data) // 2])  # inside the states: found when they are read
    from cpmd_gb300 import GbcpError
    from cpmd_gb300.restart import read_restart
    with pytest.raises(GbcpError) as e:
        read_restart(tmp_path / "trunc9")
    assert e.value.code == 9
    bad = bytearray(data)
    bad[84:88] = struct.pack("<i", 81)  # trailing frame of the header record
    (tmp_path / "frame").write_bytes(bytes(bad))
    assert _status(lib, tmp_path / "frame") == 9
    (tmp_path / "text").write_bytes(b"not a restart file" * 10)
    assert _status(lib, tmp_path / "text") == 9


def test_oversized_counts_are_reported_not_allocated(lib, tmp_path):
    """Lengths and counts read from a corrupt file are bounded by what is left
    of the file: a 2 GiB record marker or a 2^30-coefficient state count is
    reported as GBCP_ERR_IO before any buffer is sized from it."""
    na, tau0 = cell()
    c = states(64, 3, 5)
    good = tmp_path / "RESTART.good"
    RO.write(good, c, na=na, tau0=tau0, ecut=20.0, nel=6, nr=32, celldm=[10, 1, 1, 0, 0, 0])
    data = good.read_bytes()
    bad = bytearray(data)
    bad[0:4] = struct.pack("<i", 2 ** 31 - 1)  # leading frame of the first record
    (tmp_path / "huge_record").write_bytes(bytes(bad))
    assert _status(lib, tmp_path / "huge_record") == 9
    # the w_wfnio header (n, ngwks, icompr, scale): n = 3 states of ngwks = 64 coefficients
    key = struct.pack("<ii", 3, 64)
    at = data.find(key)
    assert at > 0
    bad = bytearray(data)
    bad[at + 4:at + 8] = struct.pack("<i", 2 ** 30)
    (tmp_path / "huge_states").write_bytes(bytes(bad))
    from cpmd_gb300 import GbcpError
    from cpmd_gb300.restart import read_restart
    with pytest.raises(GbcpError) as e:
        read_restart(tmp_path / "huge_states")
    assert e.value.code == 9


def test_unsupported_layouts_are_reported(lib, tmp_path):
    na, tau0 = cell()
    c = states(64, 3, 6)
    p = tmp_path / "RESTART.k"
    RO.write(p, c, na=na, tau0=tau0, ecut=20.0, nel=6, nr=32, celldm=[10, 1, 1, 0, 0, 0])
    raw = p.read_bytes()
    d = bytearray(raw)
    # section 8's record (nstate, nkpts, ngwks, ...) with k points
    body = struct.pack("<iiiiii", 3, 0, 64, 0, 0, 0)
    i = raw.index(body)
    d[i + 4:i + 8] = struct.pack("<i", 2)
    (tmp_path / "kpts").write_bytes(bytes(d))
    assert _status(lib, tmp_path / "kpts") == 7
    # section 9 in the older positive-count layout
    d = bytearray(raw)
    j = raw.index(struct.pack("<iq", -(2 * 3 + 3), -1))
    d[j:j + 4] = struct.pack("<i", 2 * 3 + 3)
    (tmp_path / "old").write_bytes(bytes(d))
    assert _status(lib, tmp_path / "old") == 7


def test_write_rejects_bad_arguments(lib, tmp_path):
    from cpmd_gb300 import GbcpError
    from cpmd_gb300.restart import write_restart
    na, tau0 = cell()
    with pytest.raises(GbcpError) as e:
        write_restart(tmp_path / "x", states(16, 2, 1), na=na, tau0=tau0, ecut=1.0, nel=2, nr=16, alat=5.0,
                      icompr=3)
    assert e.value.code == 1
    with pytest.raises(ValueError):
        write_restart(tmp_path / "y", states(16, 2, 1), na=[9], tau0=tau0, ecut=1.0, nel=2, nr=16, alat=5.0)


@pytest.mark.parametrize("stream", [False, True])
def test_occupations_and_eigenvalues(lib, tmp_path, stream):
    """Sections 23-24 after sections 10-22 that hold records the reader must skip,
    with only part of section 9's states read."""
    from cpmd_gb300.restart import read_restart, write_restart
    na, tau0 = cell(9)
    c = states(96, 7, 9)
    occ = np.array([2.0, 2.0, 2.0, 1.5, 1.0, 0.5, 0.0])
    eig = np.linspace(-0.8, 0.3, 7)
    p = tmp_path / "RESTART.occ"
    write_restart(p, c, na=na, tau0=tau0, ecut=20.0, nel=9, nr=32, alat=10.0, f=occ, eigv=eig, amu=0.125)
    ref = RO.read(p)
    assert np.array_equal(ref["f"], occ) and np.array_equal(ref["eigv"], eig) and ref["amu"] == 0.125
    d = read_restart(p, nstate=3)
    assert d.c0.shape == (96, 3) and np.array_equal(d.c0, c[:, :3])
    assert np.array_equal(d.f, occ) and np.array_equal(d.eigv, eig) and d.amu == 0.125
    assert d.has_section(23) and d.has_section(24)
    # the reference's own sections in between: accumulators (11), potential (18), density (22)
    q = tmp_path / "RESTART.fill"
    fill = {11: [b"v" * 20, b"w" * 40, b"x" * 8], 18: [b"p" * 160], 22: [b"r" * 72, b"s" * 8]}
    RO.write(q, c, na=na, tau0=tau0, ecut=20.0, nel=9, nr=32, celldm=[10, 1, 1, 0, 0, 0], f=occ, eigv=eig,
             amu=-0.25, fill=fill, stream=stream, icompr=2)
    d = read_restart(q, nstate=2)
    assert d.c0.shape == (96, 2)
    assert np.array_equal(d.c0, RO.read(q)["c0"][:, :2])
    assert np.array_equal(d.f, occ) and np.array_equal(d.eigv, eig) and d.amu == -0.25


def test_file_may_end_after_the_states(lib, tmp_path):
    from cpmd_gb300.restart import read_restart
    na, tau0 = cell()
    c = states(64, 3, 11)
    p = tmp_path / "RESTART.full"
    RO.write(p, c, na=na, tau0=tau0, ecut=20.0, nel=6, nr=32, celldm=[10, 1, 1, 0, 0, 0])
    raw = p.read_bytes()
    # cut right after section 9: the first empty section header (record of 12 bytes) follows it
    hdr10 = struct.pack("<i", 12) + struct.pack("<iq", 0, 0) + struct.pack("<i", 12)
    cut = len(raw) - 90 * len(hdr10)  # sections 10..99, all empty
    assert raw[cut:cut + len(hdr10)] == hdr10
    q = tmp_path / "RESTART.cut"
    q.write_bytes(raw[:cut])
    d = read_restart(q)
    assert np.array_equal(d.c0, c) and d.f is None and d.eigv is None


@pytest.mark.parametrize("icompr", [1, 2])
@pytest.mark.parametrize("stream", [False, True])
def test_wavefunction_velocities(lib, tmp_path, icompr, stream):
    """Section 10 (wr30wfn 'NIL', scale = largest |component|) both ways, ahead of
    sections 23-24, with fewer states read than stored."""
    from cpmd_gb300.restart import read_restart, write_restart
    na, tau0 = cell(13)
    c = states(80, 5, 13)
    cm = states(80, 5, 14) * 1e-3
    occ = np.full(5, 2.0)
    p = tmp_path / "RESTART.cm"
    if not stream:
        write_restart(p, c, na=na, tau0=tau0, ecut=20.0, nel=10, nr=32, alat=10.0, cm=cm, f=occ, icompr=icompr)
        ref = RO.read(p)
        assert ref["cm_scale"] == np.abs(np.concatenate([cm.real.ravel(), cm.imag.ravel()])).max()
        if icompr == 1:
            assert np.array_equal(ref["cm"], cm)
    else:
        RO.write(p, c, na=na, tau0=tau0, ecut=20.0, nel=10, nr=32, celldm=[10, 1, 1, 0, 0, 0], cm=cm, f=occ,
                 icompr=icompr, stream=True)
        ref = RO.read(p)
    d = read_restart(p, nstate=3)
    assert d.has_section(10) and d.cm.shape == (80, 3)
    assert np.array_equal(d.cm, ref["cm"][:, :3])
    if icompr == 1:
        assert np.array_equal(d.cm, cm[:, :3])
    else:
        assert np.abs(d.cm[:-1] - cm[:-1, :3]).max() <= ref["cm_scale"] / (2 ** 31 - 1)
    assert np.array_equal(d.f, occ)
    full = read_restart(p)
    assert full.cm.shape == (80, 5) and np.array_equal(full.cm, ref["cm"])
