"""Checkpoint files (no GPU): the reference's layout and loader contract."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from specmc_gb300 import checkpoint as ck  # noqa: E402


def test_roundtrip_and_names(tmp_path):
    that = (np.arange(12.0) + 1j * np.arange(12.0)[::-1]).reshape(3, 4)
    p = ck.save(str(tmp_path), that, 0.125, n=7, fac=40.0)
    assert os.path.basename(p) == "t_0.125000.npz" == ck.filename(ck.DEFAULT_PREFIX, 0.125)
    assert not any(f.endswith(".tmp.npz") for f in os.listdir(tmp_path))
    s, meta = ck.load(p)
    assert np.array_equal(s, that)
    assert meta["t"] == 0.125 and meta["n"] == 7 and meta["fac"] == 40.0
    assert meta["keys"] == ["fac", "n", "t", "that"] and meta["history"] is None
    ck.save(str(tmp_path), that, 0.5)
    assert [t for t, _ in ck.list_(str(tmp_path))] == [0.125, 0.5]
    assert ck.latest(str(tmp_path))[0] == 0.5
    s2, m2 = ck.load(ck.latest(str(tmp_path))[1])
    assert m2["n"] is None and m2["fac"] is None


def test_loader_errors(tmp_path):
    with pytest.raises(FileNotFoundError):
        ck.load(str(tmp_path / "missing.npz"))
    bad = tmp_path / "bad.npz"
    np.savez(bad, x=np.zeros(3))
    with pytest.raises(ValueError):
        ck.load(str(bad))


def test_files_of_the_reference_layout_load(tmp_path):
    # a file written the way specmc/io/checkpoint.py:49-56 writes it
    that = np.ones((2, 3), complex)
    fn = tmp_path / "t_0.010000.npz"
    np.savez_compressed(fn, that=that, t=0.01, n=None, fac=None)
    s, meta = ck.load(str(fn))
    assert np.array_equal(s, that) and meta["t"] == 0.01 and meta["n"] is None


def test_reference_written_checkpoint_loads_and_ours_matches_it(tmp_path):
    """A state written by the reference's own checkpoint.save
    (tests/golden/ckpt/) loads here, and save() here writes the same file name,
    keys, values and dtypes."""
    d = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ckpt")
    ref_path = os.path.join(d, "t_0.125000.npz")
    that = (np.arange(12.0) + 1j * np.arange(12.0)[::-1]).reshape(3, 4)
    s, meta = ck.load(ref_path)
    assert np.array_equal(s, that) and (meta["t"], meta["n"], meta["fac"]) == (0.125, 7, 40.0)
    assert ck.latest(d) == (0.125, ref_path)
    ours = ck.save(str(tmp_path), that, 0.125, n=7, fac=40.0)
    assert os.path.basename(ours) == os.path.basename(ref_path)
    a, b = np.load(ours, allow_pickle=True), np.load(ref_path, allow_pickle=True)
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        assert a[k].dtype == b[k].dtype and a[k].shape == b[k].shape, k
        assert np.array_equal(a[k], b[k]), k


def test_interrupted_and_corrupted_saves(tmp_path):
    """Failure injection on the host: the temporary file of an interrupted
    save, files of another prefix and names without a time are never taken
    for states; a truncated checkpoint raises instead of returning a state."""
    that = np.full((2, 3), 1.0 + 2.0j)
    good = ck.save(str(tmp_path), that, 0.25, n=3, fac=40.0)
    with open(good, "rb") as f:
        blob = f.read()
    (tmp_path / "t_0.500000.npz.tmp.npz").write_bytes(blob)      # interrupted save
    (tmp_path / "keep_0.750000.npz").write_bytes(blob)           # other prefix
    (tmp_path / "t_final.npz").write_bytes(blob)                 # no time in the name
    assert ck.list_(str(tmp_path)) == [(0.25, good)]
    assert ck.latest(str(tmp_path), ck.KEEP_PREFIX)[0] == 0.75
    cut = tmp_path / "t_1.000000.npz"
    cut.write_bytes(blob[: len(blob) // 2])                      # truncated file
    assert ck.latest(str(tmp_path))[0] == 1.0
    with pytest.raises(Exception) as err:
        ck.load(str(cut))
    assert not isinstance(err.value, AssertionError)
    assert ck.latest(str(tmp_path / "absent")) is None and ck.list_(str(tmp_path / "absent")) == []


def test_bdf2_history_roundtrip(tmp_path):
    """save(..., model=m) stores the BDF2 history the model reports;
    resume() installs it in a model, or resets the model's history for a file
    without one (a stand-in model records the calls)."""
    class Model:
        def __init__(self, have):
            self.have, self.calls = have, []

        def get_history(self):
            return dict(have_prev=self.have, prev=np.full((2, 3), 1 + 2j),
                        psi_prev=np.full((2, 3), 3j), dt_prev=2e-5)

        def set_history(self, prev, psi_prev, dt_prev, have_prev):
            self.calls.append(("set", prev.copy(), psi_prev.copy(), dt_prev, have_prev))

        def reset_history(self):
            self.calls.append(("reset",))

    s = np.arange(6.0).reshape(2, 3) + 0j
    p = ck.save(str(tmp_path), s, 1e-4, n=5, model=Model(True))
    m = Model(False)
    s2, meta = ck.resume(m, p)
    assert np.array_equal(s2, s) and meta["n"] == 5 and meta["fac"] is None
    kind, prev, psi_prev, dt_prev, have = m.calls[0]
    assert kind == "set" and have and dt_prev == 2e-5
    assert np.array_equal(prev, np.full((2, 3), 1 + 2j)) and np.array_equal(psi_prev, np.full((2, 3), 3j))
    p2 = ck.save(str(tmp_path), s, 2e-4, model=Model(False))          # no history to store
    m2 = Model(False)
    _, meta2 = ck.resume(m2, p2)
    assert meta2["history"] is None and m2.calls == [("reset",)]
