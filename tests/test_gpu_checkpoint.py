"""Checkpoint and resume: a context restored from eb_checkpoint_write continues exactly as
the uninterrupted one (no device state beyond the saved fields), and a bad file is refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "sxx", "sxy", "tk", "gii", "strain_plastic", "exx", "pr", "eta")


def test_resume_from_checkpoint_is_exact(eb, tmp_path):
    model = eb.synthetic.config("rift_small")
    a = eb.MarkerInCell(0)
    a.load_model(model)
    a.marker_cycle()
    path = tmp_path / "state.ebck"
    a.checkpoint_write(path)
    b = eb.MarkerInCell(0)
    b.set_grid(model.grid)
    b.set_materials(model.mats)
    b.set_params(model.params)
    b.checkpoint_read(path)
    assert b.marknum == model.marknum
    for mic in (a, b):
        mic.marker_cycle()
    for k in FIELDS:
        assert np.array_equal(a.download_marker(k), b.download_marker(k)), k
    for g in ("rho1", "etas1", "tk1", "dsxy"):
        assert np.array_equal(a.download_grid(g), b.download_grid(g)), g
    a.close()
    b.close()


def test_checkpoint_of_another_grid_is_refused(eb, tmp_path):
    a = eb.MarkerInCell(0)
    a.load_model(eb.synthetic.config("rift_small"))
    path = tmp_path / "state.ebck"
    a.checkpoint_write(path)
    other = eb.synthetic.config("sinking_block")
    b = eb.MarkerInCell(0)
    b.set_grid(other.grid)
    with pytest.raises(RuntimeError):
        b.checkpoint_read(path)
    (tmp_path / "junk").write_bytes(b"not a checkpoint at all")
    with pytest.raises(RuntimeError):
        b.checkpoint_read(tmp_path / "junk")
    a.close()
    b.close()


def test_truncated_checkpoint_leaves_the_context_untouched(eb, tmp_path):
    """Every entry header and size is checked before the context changes: a file cut short
    (here in its last field) is refused, and the context keeps its markers and fields."""
    a = eb.MarkerInCell(0)
    a.load_model(eb.synthetic.config("rift_small"))
    path = tmp_path / "state.ebck"
    a.checkpoint_write(path)
    data = path.read_bytes()
    cut = tmp_path / "cut.ebck"
    cut.write_bytes(data[:-100])
    b = eb.MarkerInCell(0)
    small = eb.synthetic.config("rift_small")
    b.load_model(small)
    b.marker_cycle()
    before = {k: b.download_marker(k) for k in FIELDS}
    with pytest.raises(RuntimeError, match="truncated"):
        b.checkpoint_read(cut)
    assert b.marknum == small.marknum
    for k in FIELDS:
        assert np.array_equal(b.download_marker(k), before[k]), k
    a.close()
    b.close()
