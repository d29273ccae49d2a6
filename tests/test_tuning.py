"""The launch-shape cache of woo_gb300.tuning, on the CPU with a stand-in handle."""
import json

from woo_gb300 import abi, tuning


class FakeHandle:
    def __init__(self):
        self.shape = dict(contactsBlock=128, contactsPerSM=0, cullBlock=256, integratorBlock=256, listsPerSM=0)
        self.tunes = 0
        self.closed = False

    def set_launch_shape(self, **kw):
        self.shape.update(kw)

    def autotune(self, steps):
        self.tunes += 1
        return {"shape": dict(self.shape, contactsBlock=64, cullBlock=512), "ms": 1.0, "ms_start": 1.5}

    def close(self):
        self.closed = True


def test_key_buckets():
    a = tuning.workload_key(1_000_006, abi.LAW_HERTZ_DMT)
    b = tuning.workload_key(1_100_000, abi.LAW_HERTZ_DMT)
    c = tuning.workload_key(100_000, abi.LAW_HERTZ_DMT)
    assert a == b != c
    assert "HertzDMT" in a and "box" in a
    assert tuning.workload_key(5000, abi.LAW_IDEALELPL, periodic=True) != tuning.workload_key(5000, abi.LAW_IDEALELPL)


def test_tune_once_then_cached(tmp_path):
    path = str(tmp_path / "shapes.json")
    h = FakeHandle()
    probes = []

    def probe():
        t = FakeHandle()
        probes.append(t)
        return t

    r1 = tuning.tuned(h, 0, "k", path=path, probe=probe)
    assert not r1["cached"] and len(probes) == 1 and probes[0].tunes == 1 and probes[0].closed
    assert h.tunes == 0 and h.shape["contactsBlock"] == 64 and h.shape["cullBlock"] == 512
    h2 = FakeHandle()
    r2 = tuning.tuned(h2, 0, "k", path=path, probe=probe)
    assert r2["cached"] and len(probes) == 1 and h2.shape == h.shape
    data = json.load(open(path))
    assert len(data) == 1 and list(data.values())[0]["ms"] == 1.0
    # no probe: tuned on the handle itself
    h3 = FakeHandle()
    r3 = tuning.tuned(h3, 0, "other", path=path)
    assert not r3["cached"] and h3.tunes == 1
