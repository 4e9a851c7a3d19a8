"""The on-disk H-matrix format refuses foreign files on the host, before any
device work."""
import pytest

import hmgpu


def test_foreign_file_is_refused(tmp_path):
    p = tmp_path / "x.bin"
    p.write_bytes(b"not an H-matrix at all" * 10)
    with pytest.raises(hmgpu.HMGPUError, match="not an hmgpu H-matrix file"):
        hmgpu.HMatrix.load(p)
    with pytest.raises(hmgpu.HMGPUError, match="cannot open"):
        hmgpu.HMatrix.load(tmp_path / "missing.bin")
