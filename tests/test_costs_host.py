"""Host side of the cost-term construction: the oracle's reference quirks
and the .mat loader (no GPU)."""
import numpy as np

from oracle import costs as C


def test_histogram_oracle_floor_counts_round_lookup():
    img = np.array([[0.0], [254.6], [255.0], [100.5]], np.float32)
    scrib = np.array([[1], [1], [1], [1]], np.int32)
    counts = C.histogram_counts(img, scrib, 1)[0]
    assert counts[0] == 1 and counts[254] == 1 and counts[255] == 1 and counts[100] == 1
    ct, _ = C.cost_histogram_ll(img, scrib, 1)
    # 254.6 is looked up in bin 255 (rounded), which holds one of four voxels
    assert np.isclose(ct[1, 0, 0], -np.log10(0.25 + 1e-10), rtol=1e-6)


def test_load_mat_roundtrip(tmp_path):
    from scipy.io import savemat

    from asetsmatlabmaxflow_gb300 import costs

    a = np.arange(24, dtype=np.float64).reshape(2, 3, 4, order="F")
    savemat(tmp_path / "v.mat", {"img": a, "scribbles": (a > 10).astype(np.uint8)})
    d = costs.load_mat(tmp_path / "v.mat")
    assert set(d) == {"img", "scribbles"}
    assert d["img"].dtype == np.float32 and np.array_equal(d["img"], a.astype(np.float32))
    assert d["img"].flags.f_contiguous
