"""The normal-mode transform measurement (gbrpmd_bench_nm_transform): both
forms transform correctly, and the in-register FFT that the propagator runs
keeps the state's round trip free of a systematic gain.

Bounds: forward transform against an FP64 direct sum within 1e-6 relative
(both forms); FFT round trips without a mean gain above 1e-9 per trip; the
tensor-core round trip within 1e-5 relative (it carries a small systematic
loss, reported by the benchmark)."""
import numpy as np
import pytest

from rpmd_mainz_gb300 import lib

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g

    g.build()


def test_nm_transform_forms():
    out = lib.bench_nm_transform(4096, reps=2)
    assert all(np.isfinite(v) for v in out.values())
    assert out["ms_per_transform_fft"] > 0 and out["ms_per_transform_tensor"] > 0
    assert out["forward_rel_err_fft"] < 1e-6
    assert out["forward_rel_err_tensor"] < 1e-6
    assert abs(out["gain_per_roundtrip_fft"]) < 1e-9
    assert out["roundtrip_rel_err_fft"] < 1e-6
    assert out["roundtrip_rel_err_tensor"] < 1e-5
    assert out["forward_rel_err_fft_quad"] < 1e-6
    assert abs(out["gain_per_roundtrip_fft_quad"]) < 1e-9
    assert out["roundtrip_rel_err_fft_quad"] < 1e-6
