"""The FP32 FMA probe that serves as the pair kernels' roofline denominator."""
import pytest

pytestmark = pytest.mark.gpu


def test_fp32_fma_probe(grx_lib):
    t = grx_lib.probe_fp32_fma(2000)
    # GB300: 152 SMs x 128 FMA lanes x 2 FLOP at up to 2.07 GHz = 80.5 TFLOP/s nominal
    assert 20.0 < t < 90.0
    with pytest.raises(grx_lib.GrxError):
        grx_lib.probe_fp32_fma(0)
