"""Checkpoint file framing on the host (no GPU): magic, JSON meta, 64-byte
aligned snapshot payload, atomic replacement, and rejection of foreign or
truncated files."""
import numpy as np
import pytest

from elsim_gb300 import sbm


def test_round_trip(tmp_path):
    blob = np.random.default_rng(0).integers(0, 256, size=1000, dtype=np.uint8)
    meta = {"iter": 17, "tm": 2.5e-3, "fr": 3, "note": "x" * 45}
    p = sbm.write_checkpoint(tmp_path / "a.ckpt", blob, meta)
    raw = p.read_bytes()
    assert raw[:8] == sbm.CKPT_MAGIC
    got_meta, got = sbm.read_checkpoint(p)
    assert got_meta == meta and np.array_equal(got, blob)
    assert (len(raw) - blob.size) % 64 == 0  # payload starts on a 64-byte boundary
    assert not (tmp_path / "a.ckpt.tmp").exists()


def test_overwrite_replaces_whole_file(tmp_path):
    p = tmp_path / "a.ckpt"
    sbm.write_checkpoint(p, np.zeros(5000, np.uint8), {"iter": 1})
    sbm.write_checkpoint(p, np.ones(10, np.uint8), {"iter": 2})
    meta, blob = sbm.read_checkpoint(p)
    assert meta == {"iter": 2} and blob.tolist() == [1] * 10


def test_rejects_foreign_and_truncated(tmp_path):
    p = tmp_path / "b.ckpt"
    p.write_bytes(b"NOTACKPT" + bytes(100))
    with pytest.raises(ValueError):
        sbm.read_checkpoint(p)
    q = sbm.write_checkpoint(tmp_path / "c.ckpt", np.zeros(4, np.uint8), {"k": "v" * 200})
    q.write_bytes(q.read_bytes()[:40])
    with pytest.raises(ValueError):
        sbm.read_checkpoint(q)
