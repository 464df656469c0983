"""The warm-start gain through the device kernels (see test_warmstart_gain.py
for the fixture and the CPU restatement)."""
import numpy as np
import pytest

from test_warmstart_gain import WEIGHTS, _data, _errors, _forward


@pytest.mark.gpu
def test_device_network_gains_the_same():
    """The committed weights through the device kernels (BF16 weights and
    activations) give the same proposal to within 0.1 dex on average, and the
    same gain."""
    from vulcan_gb300 import _build
    from vulcan_gb300.warmstart import MLP
    _build.build()
    w = np.load(WEIGHTS)
    X, Y, col = _data()
    m = MLP.load(WEIGHTS)
    P = m.predict(X)
    assert float(np.abs(P - _forward(w, X)).mean()) < 0.1
    e_mlp, e_eq, e_cm = _errors(P, X, Y, col)
    assert e_mlp < 0.25 and e_mlp < 0.3 * e_eq < e_cm
