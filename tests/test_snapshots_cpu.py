"""snapshot! and restart_from_height host side (src/measures.jl:99-105,
src/initialvalues.jl:358-382), with the reference's test numbers
(test/measures.jl:122-130 and the restart doctest)."""
import numpy as np

import swalbe_gb300 as sw


def test_snapshot_like_reference():
    h1 = np.arange(1, 26).reshape(5, 5, order="F")
    h2 = np.arange(5, 126, 5).reshape(5, 5, order="F")
    snap = np.zeros((2, 25))
    sw.snapshot_(snap, h1, 10, dumping=10)
    sw.snapshot_(snap, h2, 20, dumping=10)
    sw.snapshot_(snap, h2 * 0, 15, dumping=10)  # not a dump step
    assert np.all(h1 == snap[0].reshape(5, 5, order="F"))
    assert np.all(h2 == snap[1].reshape(5, 5, order="F"))


def test_restart_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    h1, h2 = rng.random((10, 10)), rng.random((10, 10))
    path = str(tmp_path / "file.npz")
    sw.save_snapshots(path, [1, 2], [h1.ravel(order="F"), h2.ravel(order="F")])
    assert np.all(sw.restart_from_height(path, timestep=1, size=(10, 10)) == h1)
    assert np.all(sw.restart_from_height(path, size=(10, 10)) == h2)  # timestep 0: the last
