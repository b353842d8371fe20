"""The FMA throughput probe the bench reports beside the HBM roofline: a
positive rate in the range a GB300 can give (FP32 FMA at most 152 SMs x 128
lanes x 2 flops x ~2.1 GHz, about 82 TFLOP/s; FP64 far below it)."""
import math

import pytest

pytestmark = pytest.mark.gpu


def test_fma_probe(hc, ctx):
    f32 = hc.measure_fma("f32")
    f64 = hc.measure_fma("f64")
    assert math.isfinite(f32) and 5.0 < f32 < 100.0, f32
    assert math.isfinite(f64) and 0.0 < f64 < f32, f64
    assert hc.load_library().hc_measure_fma(7, None) == -1     # HC_ERR_INVALID
