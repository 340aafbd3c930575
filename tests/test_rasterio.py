"""Raster files to and from device memory (the I/O step before the path).

The .npy header parser runs on the CPU; the transfers run on the GPU and
must return the file's bytes unchanged, for Fortran- and C-order files,
across chunk boundaries (the 16 MiB staging chunks), at an offset, and for
a round trip through write_npy.
"""
import numpy as np
import pytest


def test_npy_header(tmp_path):
    from libtopotoolbox_gb300 import rasterio

    a = np.asfortranarray(np.arange(12, dtype=np.float32).reshape(3, 4))
    np.save(tmp_path / "a.npy", a)
    descr, fortran, shape, off = rasterio.npy_header(tmp_path / "a.npy")
    assert (descr, fortran, shape) == ("<f4", True, (3, 4))
    raw = (tmp_path / "a.npy").read_bytes()
    assert np.array_equal(np.frombuffer(raw[off:], np.float32), a.ravel(order="F"))


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(5, 7), (2049, 3001), (4096, 4097)])
def test_read_npy_roundtrip(gpu, tmp_path, shape):
    from libtopotoolbox_gb300 import rasterio

    rng = np.random.default_rng(shape[0])
    a = rng.standard_normal(shape).astype(np.float32)
    np.save(tmp_path / "f.npy", np.asfortranarray(a))
    np.save(tmp_path / "c.npy", np.ascontiguousarray(a))
    for name in ("f.npy", "c.npy"):
        t = rasterio.read_npy(tmp_path / name)
        assert tuple(t.shape) == (shape[1], shape[0])
        assert np.array_equal(t.cpu().numpy().T, a), name
    rasterio.write_npy(tmp_path / "w.npy", rasterio.read_npy(tmp_path / "f.npy"))
    back = np.load(tmp_path / "w.npy")
    assert back.flags.f_contiguous and np.array_equal(back, a)


@pytest.mark.gpu
def test_read_raw_offset_and_errors(gpu, tmp_path):
    from libtopotoolbox_gb300 import _native, rasterio

    torch = gpu
    data = np.arange(40 << 20, dtype=np.uint8)  # crosses two staging chunks
    (tmp_path / "r.bin").write_bytes(b"HEADER" + data.tobytes())
    t = rasterio.read_raw(tmp_path / "r.bin", 6, (data.size,), torch.uint8)
    assert np.array_equal(t.cpu().numpy(), data)
    with pytest.raises(_native.TTCudaError) as e:
        rasterio.read_raw(tmp_path / "missing.bin", 0, (4,), torch.uint8)
    assert e.value.status == 7
    with pytest.raises(_native.TTCudaError) as e:  # file shorter than asked
        rasterio.read_raw(tmp_path / "r.bin", 6, (data.size + 1,), torch.uint8)
    assert e.value.status == 7
