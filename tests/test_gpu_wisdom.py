"""Plan wisdom on the GPU: a tuned plan's record rebuilds the same plan
without timing, with bit-identical results, and a record that no longer
fits its plan is replaced by a fresh tuning."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plan(precision):
    from fftwpp_gb300.gpu import HybridConvolution, CENTERED, HERMITIAN
    return HybridConvolution([CENTERED, HERMITIAN], [63, 63],
                             precision=precision)


def _schedule(conv):
    return (conv.axes, conv.rows_per_cta, conv.threads_per_cta)


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_wisdom_rebuilds_plan(native_lib, precision):
    import torch
    from fftwpp_gb300 import gpu
    gpu.forget_wisdom()
    try:
        a = _plan(precision)
        text = gpu.export_wisdom()
        assert text.count("\n") == 1 and text.startswith("fgb1 ")
        gpu.forget_wisdom()
        assert gpu.import_wisdom(text) == 1
        b = _plan(precision)
        assert gpu.export_wisdom() == text
        assert _schedule(a) == _schedule(b)
        rng = np.random.default_rng(5)
        shape = (63, 32)
        fs = [torch.from_numpy(rng.standard_normal(shape) +
                               1j * rng.standard_normal(shape))
              .to(a.dtype).cuda() for _ in range(2)]
        ra = a.convolve(*fs)[0].cpu().numpy()
        rb = b.convolve(*fs)[0].cpu().numpy()
        assert np.array_equal(ra, rb)
    finally:
        gpu.forget_wisdom()


def test_wisdom_record_that_does_not_fit(native_lib):
    from fftwpp_gb300 import gpu
    gpu.forget_wisdom()
    try:
        _plan("f64")
        key, value = gpu.export_wisdom().rstrip("\n").split("\t")
        v = value.split()
        v[3] = "16"                       # x column tile 16: over the FP64 cap
        gpu.forget_wisdom()
        gpu.import_wisdom(f"{key}\t{' '.join(v)}\n")
        c = _plan("f64")
        new = gpu.export_wisdom().rstrip("\n").split("\t")[1].split()
        assert new[3] != "16"
        assert c.axes[0]["tile"] == int(new[3])
    finally:
        gpu.forget_wisdom()
