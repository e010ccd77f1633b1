"""The product path has no CPU fallback: without the native library, or given host arrays, the
calls fail loudly instead of computing anything (no GPU needed to check)."""
import pytest

torch = pytest.importorskip("torch")


def test_missing_native_library_raises(monkeypatch, tmp_path):
    from pelelm_gb300 import _lib
    monkeypatch.setattr(_lib, "LIB", str(tmp_path / "libpelelm_gb300.so"))
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="native library missing"):
        _lib.lib()


def test_host_arrays_are_refused():
    from pelelm_gb300.reactor import array4
    with pytest.raises(ValueError, match="CUDA tensors"):
        array4(torch.zeros(3, 4, 4, 4, dtype=torch.float64))


def test_box_views_need_contiguous_i_and_four_dimensions():
    from pelelm_gb300.reactor import array4

    class FakeCuda:
        """Shape/stride stand-in for a CUDA tensor (array4 only reads its metadata)."""
        is_cuda = True

        def __init__(self, shape, stride):
            self.shape, self._stride = shape, stride

        def dim(self):
            return len(self.shape)

        def stride(self):
            return self._stride

        def data_ptr(self):
            return 4096

    with pytest.raises(ValueError, match="contiguous"):
        array4(FakeCuda((2, 4, 4, 4), (64, 16, 4, 2)))
    with pytest.raises(ValueError, match="nz, ny, nx"):
        array4(FakeCuda((2, 2, 4, 4, 4), (128, 64, 16, 4, 1)))
    a = array4(FakeCuda((3, 5, 6, 7), (210, 42, 7, 1)), lo=(-2, 10, 4))
    assert (a.jstride, a.kstride, a.nstride, a.ncomp) == (7, 42, 210, 3)
    assert tuple(a.begin) == (-2, 10, 4) and tuple(a.end) == (5, 16, 9)  # end exclusive, as Array4
