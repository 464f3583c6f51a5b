"""Checkpoint / resume of a grid of geometries (cipsi_gb300.batch.run_grid):
each geometry's result is saved as its batch finishes, and a run that
stopped continues with the geometries that have no result, as the Autocip
driver re-reads finished geometries.  The batched launch itself is replaced
by a stand-in here (it needs a GPU; the batched form is checked against the
plain one in test_gpu_batch)."""
import json
import os

import pytest

from cipsi_gb300 import batch, synth


class Runner:
    """Stand-in for run_batch: a result per geometry, optionally failing at
    a given call, recording which geometries each call got."""

    def __init__(self, fail_at=None):
        self.calls = []
        self.fail_at = fail_at

    def __call__(self, cfgs, **kw):
        self.calls.append([c.name for c in cfgs])
        if self.fail_at is not None and len(self.calls) == self.fail_at:
            raise RuntimeError("batch failed")
        return [{"e2vp": [float(c.seed) + 0.5], "ncf": c.ncf} for c in cfgs]


def test_stopped_grid_resumes_with_the_unfinished_geometries(tmp_path):
    cfgs = synth.curve_geometries(10, seed=5)
    out = str(tmp_path / "res")
    first = Runner(fail_at=2)
    with pytest.raises(RuntimeError, match="batch failed"):
        batch.run_grid(cfgs, out, batch_size=4, runner=first)
    done = sorted(f for f in os.listdir(out))
    assert done == sorted(c.name + ".json" for c in cfgs[:4])  # the first batch only
    # a write cut short leaves only a temporary file, which is not a result
    with open(os.path.join(out, cfgs[5].name + ".json.tmp"), "w") as fh:
        fh.write("{")
    second = Runner()
    res = batch.run_grid(cfgs, out, batch_size=4, runner=second)
    assert second.calls == [[c.name for c in cfgs[4:8]], [c.name for c in cfgs[8:]]]
    assert set(res) == {c.name for c in cfgs}
    for c in cfgs:
        assert res[c.name] == {"e2vp": [float(c.seed) + 0.5], "ncf": c.ncf}
        rec = json.load(open(os.path.join(out, c.name + ".json")))
        assert (rec["norb"], rec["ncf"], rec["curve_R"]) == (c.norb, c.ncf, c.curve_R)
    # nothing left to run
    third = Runner()
    assert batch.run_grid(cfgs, out, batch_size=4, runner=third) == res and third.calls == []


def test_grid_refuses_duplicate_names_and_short_batches(tmp_path):
    cfgs = synth.curve_geometries(3, seed=6)
    with pytest.raises(ValueError, match="unique"):
        batch.run_grid(cfgs + cfgs[:1], str(tmp_path / "a"), runner=Runner())
    with pytest.raises(RuntimeError, match="results"):
        batch.run_grid(cfgs, str(tmp_path / "b"), runner=lambda cs, **kw: [{}])


def test_grid_reruns_results_of_another_configuration(tmp_path):
    # the same geometry names (geo000, geo001, ...) with another seed in the
    # same directory: the saved results belong to other systems
    out = str(tmp_path / "res")
    old = synth.curve_geometries(4, seed=5)
    batch.run_grid(old, out, batch_size=4, runner=Runner())
    new = synth.curve_geometries(4, seed=7)
    assert [c.name for c in new] == [c.name for c in old]
    assert any((a.seed, a.norb, a.curve_R) != (b.seed, b.norb, b.curve_R) for a, b in zip(old, new))
    second = Runner()
    res = batch.run_grid(new, out, batch_size=4, runner=second)
    changed = [b.name for a, b in zip(old, new) if any(getattr(a, f) != getattr(b, f) for f in batch._KEY_FIELDS)]
    assert second.calls == [changed]
    for c in new:
        assert res[c.name] == {"e2vp": [float(c.seed) + 0.5], "ncf": c.ncf}
        assert json.load(open(os.path.join(out, c.name + ".json")))["seed"] == c.seed


def test_grid_reruns_a_result_file_that_does_not_parse(tmp_path):
    out = str(tmp_path / "res")
    cfgs = synth.curve_geometries(3, seed=5)
    batch.run_grid(cfgs, out, batch_size=3, runner=Runner())
    # a renamed file whose data never reached the disk (power loss)
    with open(os.path.join(out, cfgs[1].name + ".json"), "w") as fh:
        fh.write('{"name": "geo0')
    second = Runner()
    res = batch.run_grid(cfgs, out, batch_size=3, runner=second)
    assert second.calls == [[cfgs[1].name]]
    assert res[cfgs[1].name] == {"e2vp": [float(cfgs[1].seed) + 0.5], "ncf": cfgs[1].ncf}
