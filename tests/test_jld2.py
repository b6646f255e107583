"""JLD2 solution files (File/save.jl, File/load.jl): the HDF5 subset the
writer emits, read back by the module's reader, the Jenkins lookup3
checksum against its published test vectors, and the reader against a
file written by libhdf5 itself (scipy's MATLAB 7.3 test file)."""
import os
import struct

import numpy as np
import pytest


@pytest.fixture(scope="module")
def J(pkg):
    return pkg.jld2


def test_lookup3_published_vectors(J):
    # lookup3.c (Bob Jenkins, 2006), driver5
    assert J.lookup3(b"", 0) == 0xDEADBEEF
    assert J.lookup3(b"", 0xDEADBEEF) == 0xBD5B7DDE
    s = b"Four score and seven years ago"
    assert J.lookup3(s, 0) == 0x17770551
    assert J.lookup3(s, 1) == 0xCD628161


def test_round_trip(J, tmp_path):
    rng = np.random.default_rng(7)
    rec = {"u": rng.standard_normal((6, 4, 15)), "t": 0.125, "du": rng.standard_normal((6, 4, 15)),
           "steps": np.array([0, 2, 4], dtype=np.int64), "empty": np.zeros(0, dtype=np.int64),
           "f32": rng.standard_normal(7).astype(np.float32), "i32": np.arange(5, dtype=np.int32),
           "n": np.int64(42), "name": "EulerEquations{2}"}
    f = str(tmp_path / "r.jld2")
    J.save(f, rec)
    back = J.load(f)
    assert set(back) == set(rec)
    for k in ("u", "du", "steps", "empty", "f32", "i32"):
        assert back[k].dtype == rec[k].dtype and back[k].shape == rec[k].shape
        assert np.array_equal(back[k], rec[k])
    assert back["t"] == 0.125 and isinstance(back["t"], float)
    assert back["n"] == 42
    assert back["name"] == "EulerEquations{2}"


def test_file_structure(J, tmp_path):
    """JLD2 header, version-2 superblock at 512 with base address 512 and the
    absolute end-of-file address, and the array's bytes stored contiguously
    in the reference's column-major order at the address its layout gives."""
    u = np.arange(2 * 3 * 5, dtype=np.float64).reshape(2, 3, 5)   # Julia (5, 3, 2)
    f = str(tmp_path / "s.jld2")
    J.save(f, {"u": u, "t": 1.5})
    buf = open(f, "rb").read()
    assert buf.startswith(b"HDF5-based Julia Data Format, version ")
    sb = 512
    assert buf[sb:sb + 8] == J.HDF5_SIGNATURE and buf[sb + 8] == 2
    base, ext, eof, root = struct.unpack_from("<QQQQ", buf, sb + 12)
    assert base == 512 and ext == J.UNDEF and eof == len(buf)
    assert struct.unpack_from("<I", buf, sb + 44)[0] == J.lookup3(buf[sb:sb + 44])
    fr = J._File(buf)
    links = fr.links(root)
    assert sorted(links) == ["t", "u"]
    msgs = dict(fr.messages(links["u"]))
    assert fr._dataspace(msgs[J.MSG_DATASPACE]) == (2, 3, 5)
    lay = msgs[J.MSG_LAYOUT]
    assert lay[0] == 3 and lay[1] == 1           # version 3, contiguous
    addr, size = struct.unpack_from("<QQ", lay, 2)
    assert size == u.nbytes
    assert buf[512 + addr:512 + addr + size] == u.tobytes()
    # the scalar time is compact
    assert dict(fr.messages(links["t"]))[J.MSG_LAYOUT][1] == 0


def test_checksums_detect_corruption(J, tmp_path):
    f = str(tmp_path / "c.jld2")
    J.save(f, {"u": np.ones((3, 3)), "t": 0.0})
    buf = bytearray(open(f, "rb").read())
    buf[512 + 48 + 10] ^= 0x40                   # inside the root group's object header
    open(f, "wb").write(bytes(buf))
    with pytest.raises(J.FormatError):
        J.load(f)
    buf[512 + 48 + 10] ^= 0x40
    buf[512 + 20] ^= 0x01                        # the superblock's end-of-file address
    open(f, "wb").write(bytes(buf))
    with pytest.raises(J.FormatError):
        J.load(f)


def test_reads_a_file_written_by_libhdf5(J):
    """scipy ships a MATLAB 7.3 file, i.e. HDF5 written by libhdf5 (512-byte
    user block, superblock version 0, symbol-table group, layout version 2):
    its variable testdouble is pi/4 (0, 1, ..., 8) as a 1 x 9 MATLAB row,
    stored column-major with the dimensions reversed."""
    sio = pytest.importorskip("scipy.io")
    f = os.path.join(os.path.dirname(sio.__file__), "matlab", "tests", "data", "testhdf5_7.4_GLNX86.mat")
    if not os.path.exists(f):
        pytest.skip("scipy's MATLAB 7.3 test file is not installed")
    d = J.load(f)
    assert list(d) == ["testdouble"]
    assert d["testdouble"].shape == (9, 1)
    assert np.allclose(d["testdouble"].ravel(), np.pi / 4 * np.arange(9), rtol=0, atol=1e-15)


def test_project_solutions_snapshots(J, pkg, tmp_path):
    """save_project / save_solution / load_time_steps / load_solution /
    load_snapshots(_with_derivatives) (File/save.jl:22-81, File/load.jl)."""
    pb = pkg.setups.vortex_tri(cells=2, p=2)
    h = pb.host_arrays()
    root = str(tmp_path / "results") + "/"
    path = J.save_project(pb, (0.0, 1.0), root)
    assert path == root
    assert list(J.load_time_steps(path)) == []
    proj = J.load_project(path)
    assert (int(proj["N_p"]), int(proj["N_c"]), int(proj["N_e"])) == (h.N_p, h.N_c, h.N_e)
    assert np.array_equal(proj["tspan"], [0.0, 1.0])
    assert "EulerEquations" in proj["conservation_law"]
    rng = np.random.default_rng(3)
    us = {s: pb.u0 + 1e-3 * rng.standard_normal(pb.u0.shape) for s in (0, 2, 4)}
    dus = {s: rng.standard_normal(pb.u0.shape) for s in us}
    for s in us:
        J.save_solution(us[s], 0.1 * s, path, s, dus[s])
    assert list(J.load_time_steps(path)) == [0, 2, 4]
    u, t = J.load_solution(path, 2)
    assert np.array_equal(u, us[2]) and t == pytest.approx(0.2)
    u, du, t = J.load_solution(path, 4, load_du=True)
    assert np.array_equal(du, dus[4])
    X, ts = J.load_snapshots(path, [0, 2, 4])
    assert X.shape == (h.N_p * h.N_c * h.N_e, 3)
    assert np.array_equal(X[:, 1], us[2].reshape(-1)) and ts == pytest.approx(0.2)
    U, dU, ts = J.load_snapshots_with_derivatives(path, [0, 2, 4])
    assert np.array_equal(dU[:, 2], dus[4].reshape(-1))
    # an existing results directory is not overwritten unless asked
    other = J.save_project(pb, (0.0, 1.0), root)
    assert other.rstrip("/") == root.rstrip("/") + "_1"
    again = J.save_project(pb, (0.0, 1.0), root, overwrite=True, clear=True)
    assert again == root and list(J.load_time_steps(again)) == []
