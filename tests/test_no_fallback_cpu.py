"""The product has no CPU fallback: without its CUDA library it refuses to
load, and without a GPU every entry point that computes reports a CUDA error
instead of computing on the host."""
import numpy as np
import pytest

import molds_gb300 as M


def test_missing_library_raises(tmp_path, monkeypatch):
    monkeypatch.setattr(M, "_lib", None)   # another test may have loaded the built library already
    with pytest.raises(ImportError, match="no CPU fallback"):
        M.load_library(str(tmp_path / "libnddo_gb300.so"))


def _gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except ImportError:
        return False


@pytest.mark.skipif(_gpu_present(), reason="a GPU is present: the GPU tests cover the computing paths")
def test_no_gpu_is_an_error_not_a_host_computation():
    from molds_gb300 import build
    build.build()
    with pytest.raises(M.NddoError) as e:
        M.Context(0)
    assert e.value.code == M.ERR_CUDA
    water = M.Molecule(np.array([8, 1, 1], dtype=np.int32),
                       np.array([[0.0, 0.0, 0.0], [1.8, 0.0, 0.0], [-0.45, 1.75, 0.0]]))
    with pytest.raises(M.NddoError):
        M.batch_scf("pm3", [water])
