"""Scene input and frame output in the reference's formats (no GPU): the OBJ reader
(wavefront.h:12-67), the .SIM writer/reader (examples/src/utils.h:29-40), Frame::fft
(radar.h:412-435) and Frame::argmax (radar.h:534-546)."""
import numpy as np

from hussar_gb300 import Frame, FrameConfig, TriangleMesh
from hussar_gb300.io import WavefrontFile, read_sim, save_frame, write_frame
from hussar_gb300.radar import complex_abs

OBJ = """# a unit quad and a triangle
v 0 0 0
v 1 0 0
v 1 1 0 1.0
v 0 1 0
vn 0 0 1
s off
f 1 2 3
f 1 3 4 2

f 1/1/1 2/2/2 4/4/4
"""


def test_wavefront_reads_like_the_reference(tmp_path):
    p = tmp_path / "quad.obj"
    p.write_text(OBJ)
    m = TriangleMesh()
    m.addQuad([5, 5, 5], [1, 0, 0], [0, 1, 0])  # 4 vertices already present
    rd = WavefrontFile(str(p))
    rd.read(m)
    v, f = m.vertexBuffer, m.indexBuffer
    assert v.shape == (8, 3) and np.array_equal(v[4:], np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32))
    # 1-based indices counted from the vertices the mesh had before the read
    assert np.array_equal(f[2:], np.array([[4, 5, 6], [4, 6, 7], [4, 5, 7]]))
    assert rd.unsupported == ["vn"]
    # a second read appends again, offset by the eight vertices now present
    WavefrontFile(str(p)).read(m)
    assert m.vertexBuffer.shape == (12, 3) and np.array_equal(m.indexBuffer[5], [8, 9, 10])


def test_sim_file_layout_and_round_trip(tmp_path):
    cfg = FrameConfig(2, 8, 3)
    rng = np.random.default_rng(0)
    frames = []
    path = tmp_path / "poses.SIM"
    with open(path, "wb") as fh:
        for _ in range(4):  # one frame per pose, appended (1_dihedral.cpp:87-126)
            f = Frame(cfg)
            f.data[...] = (rng.normal(size=f.data.shape) + 1j * rng.normal(size=f.data.shape)).astype(np.complex64)
            write_frame(fh, f)
            frames.append(f.data.copy())
    raw = np.fromfile(path, np.float32)
    # element i of frame 0 is (re, im) at float offset 2 i, in [chirp][sample][channel] order
    assert raw[0] == frames[0][0, 0, 0].real and raw[1] == frames[0][0, 0, 0].imag
    assert raw[2] == frames[0][0, 0, 1].real
    back = read_sim(str(path), cfg)
    assert back.shape == (4, 2, 8, 3) and np.array_equal(back, np.stack(frames))
    save_frame(Frame(cfg), str(tmp_path / "one"))
    assert (tmp_path / "one.SIM").stat().st_size == 8 * cfg.sampleCount()


def test_frame_fft_is_the_unnormalised_forward_3d_dft():
    cfg = FrameConfig(2, 5, 3)
    rng = np.random.default_rng(1)
    f = Frame(cfg)
    x = (rng.normal(size=f.data.shape) + 1j * rng.normal(size=f.data.shape)).astype(np.complex64)
    f.data[...] = x
    f.fft()
    # direct sum: X[k] = sum_n x[n] exp(-2 pi i sum_a k_a n_a / N_a)
    C, S, H = x.shape
    n = np.stack(np.meshgrid(np.arange(C), np.arange(S), np.arange(H), indexing="ij"), -1).reshape(-1, 3)
    ph = -2j * np.pi * (np.outer(n[:, 0], n[:, 0]) / C + np.outer(n[:, 1], n[:, 1]) / S + np.outer(n[:, 2], n[:, 2]) / H)
    ref = (np.exp(ph) @ x.reshape(-1).astype(np.complex128)).reshape(x.shape)
    assert np.allclose(f.data, ref, rtol=1e-5, atol=1e-5)


def test_argmax_first_of_equal_magnitudes_and_reference_abs():
    f = Frame(FrameConfig(1, 6, 2))
    f.data[0, 2, 1] = 3 + 4j
    f.data[0, 4, 0] = -4 + 3j  # same magnitude, later index
    assert tuple(int(i) for i in f.argmax()) == (0, 2, 1)
    z = np.array([3 + 4j, 0, 1e-30 + 1e-30j, -2.5 - 0j], np.complex64)
    a = complex_abs(z)
    assert a.dtype == np.float32 and a[0] == np.float32(5) and a[1] == 0 and a[3] == np.float32(2.5)
    assert np.isclose(a[2], np.float32(np.sqrt(2) * 1e-30), rtol=1e-6)


def test_native_obj_reader_matches_python_reader(tmp_path, product_lib):
    """hsr_read_obj (the C ABI's WavefrontFile::read, host only) gives the Python reader's
    vertices and indices, offset by the caller's vertex count, and counts the skipped
    commands; a short face line is an error."""
    import ctypes
    from hussar_gb300 import _lib
    p = tmp_path / "quad.obj"
    p.write_text(OBJ)
    L = product_lib
    nv, nt, un = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    _lib.check(L.hsr_read_obj(str(p).encode(), 4, None, 0, None, 0, ctypes.byref(nv), ctypes.byref(nt),
                              ctypes.byref(un)))
    assert (nv.value, nt.value, un.value) == (4, 3, 1)
    v = np.zeros((nv.value, 3), np.float32)
    f = np.zeros((nt.value, 3), np.int32)
    _lib.check(L.hsr_read_obj(str(p).encode(), 4, v.ctypes.data, nv.value, f.ctypes.data, nt.value,
                              ctypes.byref(nv), ctypes.byref(nt), None))
    m = TriangleMesh()
    m.addQuad([5, 5, 5], [1, 0, 0], [0, 1, 0])
    WavefrontFile(str(p)).read(m)
    assert np.array_equal(v, m.vertexBuffer[4:]) and np.array_equal(f, m.indexBuffer[2:])
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nf 1 1\n")
    st = L.hsr_read_obj(str(bad).encode(), 0, None, 0, None, 0, ctypes.byref(nv), ctypes.byref(nt), None)
    assert st == _lib.HSR_ERR_INVALID_ARGUMENT
    st = L.hsr_read_obj(str(tmp_path / "missing.obj").encode(), 0, None, 0, None, 0, ctypes.byref(nv),
                        ctypes.byref(nt), None)
    assert st == _lib.HSR_ERR_INVALID_ARGUMENT
