"""Moment files: binary round trips with the header fields, checksum and
format errors; the reference's text layouts (TB/utils.h:42-69,
TB/snippets.h:504-517).  Host only."""
import numpy as np
import pytest


def test_binary_round_trips(tb, tmp_path):
    rng = np.random.default_rng(0)
    mu = rng.standard_normal(1024)
    p = tmp_path / "dos.tbm"
    tb.save_moments(p, mu, kind="dos", R=32, seed=7, e_min=-8.6, e_max=8.6, precision=2, kernel=3,
                    n_sites=2097152, label="honeycomb 1024x1024 W=1")
    got, meta = tb.load_moments(p)
    assert np.array_equal(got, mu)
    assert meta["kind"] == "dos" and meta["R"] == 32 and meta["seed"] == 7 and meta["precision"] == 2
    assert meta["e_min"] == -8.6 and meta["kernel"] == 3 and meta["n_sites"] == 2097152
    assert meta["label"] == "honeycomb 1024x1024 W=1"
    assert p.stat().st_size == 256 + 8 * 1024
    m = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
    tb.save_moments(tmp_path / "mu.tbm", m, kind="mu_nm", R=4)
    got, meta = tb.load_moments(tmp_path / "mu.tbm")
    assert np.array_equal(got, m) and meta["kind"] == "mu_nm"
    V = np.triu(rng.standard_normal((16, 16)))
    tb.save_moments(tmp_path / "v.tbm", V, kind="v_nm")
    assert np.array_equal(tb.load_moments(tmp_path / "v.tbm")[0], V)


def test_binary_errors(tb, tmp_path):
    p = tmp_path / "dos.tbm"
    tb.save_moments(p, np.arange(10.0))
    raw = bytearray(p.read_bytes())
    raw[256 + 13] ^= 0x40
    (tmp_path / "flip.tbm").write_bytes(bytes(raw))
    with pytest.raises(tb.TbkError, match="checksum mismatch"):
        tb.load_moments(tmp_path / "flip.tbm")
    (tmp_path / "short.tbm").write_bytes(p.read_bytes()[:300])
    with pytest.raises(tb.TbkError, match="short moment file"):
        tb.load_moments(tmp_path / "short.tbm")
    (tmp_path / "magic.tbm").write_bytes(b"X" + p.read_bytes()[1:])
    with pytest.raises(tb.TbkError, match="bad magic"):
        tb.load_moments(tmp_path / "magic.tbm")
    with pytest.raises(tb.TbkError, match="Fail to open"):
        tb.load_moments(tmp_path / "missing.tbm")


def test_text_layouts(tb, tmp_path):
    f = tmp_path / "dos.txt"
    tb.output_to_file(f, [0.1, -2.0, 1e-7], [3.0, 4.123456789, 0.0])
    assert f.read_text() == "0.1 3 \n-2 4.12346 \n1e-07 0 \n"
    with pytest.raises(ValueError, match="Not equal size"):
        tb.output_to_file(f, [1.0], [1.0, 2.0])
    v = tmp_path / "V_moments.txt"
    tb.write_V_moments_text(v, np.array([[1.5, 2.0, -3.0], [9.0, 0.25, 1e-9], [9.0, 9.0, 7.0]]))
    assert v.read_text() == "1.5 2 -3 \n0 0.25 1e-09 \n0 0 7 \n"
