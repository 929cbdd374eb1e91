"""CPU tests of the reference file formats (survival dumps, Chebyshev checkpoint)."""
import numpy as np

from dynemol_gb300 import io


def test_survival_format(tmp_path):
    w = io.SurvivalWriter(str(tmp_path), "el", ["D", "A"])
    w.write(0.0001, [0.64590519, 0.35409481, 1.0], 1.5 - 0.25j)
    w.write(0.0002, [0.5, 0.5, 1.0], 1.5 - 0.25j)
    lines = open(tmp_path / "el_survival.dat").read().splitlines()
    assert lines[0] == "#        1         2         3         4"
    assert lines[1] == ""
    assert lines[2] == "         #         D         A     total"
    assert lines[3] == "   0.000100   0.64591   0.35409   1.00000"
    data = io.read_survival(str(tmp_path / "el_survival.dat"))
    assert data.shape == (2, 4)
    assert open(tmp_path / "el_wp_energy.dat").read().splitlines()[0] == "    0.000100    1.500000   -0.250000"


def test_checkpoint_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    N, P = 7, 2
    cz = lambda: rng.normal(size=(N, P)) + 1j * rng.normal(size=(N, P))
    db, dk, ab, ak = cz(), cz(), cz(), cz()
    q = rng.normal(size=3)
    path = str(tmp_path / "Security_copy.dat")
    io.write_checkpoint(path, 17, 0.0123, db, dk, ab, ak, charges=q, frame=5)
    ck = io.read_checkpoint(path, with_frame=True)
    assert ck["frame"] == 5 and ck["it"] == 17 and ck["t"] == 0.0123 and ck["tags"] == ["el", "hl"]
    for k, v in (("dual_bra", db), ("dual_ket", dk), ("ao_bra", ab), ("ao_ket", ak)):
        assert np.array_equal(ck[k], v)
    assert np.array_equal(ck["net_charge"], q)
    # record markers: first record is the 4-byte frame
    raw = open(path, "rb").read()
    assert raw[:4] == (4).to_bytes(4, "little") and raw[8:12] == (4).to_bytes(4, "little")
    b, k = io.state_from_checkpoint(ck)
    assert np.array_equal(b, dk) and np.array_equal(k, ak)
