"""Coefficient table persistence: a table saved by one interpolant loads into
a fresh interpolant of the same field and gives identical table queries;
files from another field, mode or precision are refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_save_load_roundtrip(prec, tmp_path):
    from arbinterp_gb300 import tricubic, synth
    f = synth.dipole_field3(n=(20, 18, 16), seed=4).numpy()
    a = tricubic(f, "quiet", mode="both", precision=prec, strategy="table")
    path = str(tmp_path / "coef.npz")
    a.save_coefficients(path)
    b = tricubic(f, "quiet", mode="both", precision=prec, strategy="table")
    b.load_coefficients(path)
    assert b._table_complete
    q = np.random.default_rng(0).uniform(a._lo, a._hi, (2000, 3))
    for x, y in zip(a.Query(q.copy()), b.Query(q.copy())):
        assert np.array_equal(x, y, equal_nan=True)
    assert np.array_equal(a.alphan, b.alphan, equal_nan=True)


def test_load_refuses_other_fields(tmp_path):
    from arbinterp_gb300 import tricubic, synth
    f = synth.dipole_field3(n=(20, 18, 16), seed=4).numpy()
    path = str(tmp_path / "coef.npz")
    tricubic(f, "quiet", mode="both").save_coefficients(path)
    g = f.copy()
    g[100, 3] += 1e-3                                  # same geometry, one value changed
    with pytest.raises(ValueError):
        tricubic(g, "quiet", mode="both").load_coefficients(path)
    with pytest.raises(ValueError):
        tricubic(f, "quiet", mode="norm").load_coefficients(path)
    with pytest.raises(ValueError):
        tricubic(f, "quiet", mode="both", precision="mixed").load_coefficients(path)
