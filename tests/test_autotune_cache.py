"""The autotuner's JSON cache on the host: save / load per device name and key
size, replace-whole writes under a lock, concurrent savers keep each other's
entries, and a damaged file reads as empty."""

import threading

from heu_gb300 import autotune


def test_save_and_load_round_trip(tmp_path):
    path = str(tmp_path / "sub" / "tuning.json")
    cfg = {"variant": 1, "dec_variant": 0, "mul_window": 4, "dec_window": 6}
    autotune.save(cfg, 2048, path=path, rates={"encrypt": 1.0})
    autotune.save(dict(cfg, variant=0), 3072, path=path)
    assert autotune.load(2048, path=path) == cfg
    assert autotune.load(3072, path=path)["variant"] == 0
    assert autotune.load(1024, path=path) is None
    left = sorted(p.name for p in (tmp_path / "sub").iterdir())
    assert left == ["tuning.json", "tuning.json.lock"]  # no temporary left behind
    (tmp_path / "sub" / "tuning.json").write_text("{not json")
    assert autotune.load(2048, path=path) is None
    autotune.save(cfg, 2048, path=path)
    assert autotune.load(2048, path=path) == cfg


def test_concurrent_saves_keep_every_entry(tmp_path):
    path = str(tmp_path / "tuning.json")
    sizes = list(range(1024, 1024 + 64 * 24, 64))

    def worker(bits):
        for _ in range(5):
            autotune.save({"variant": bits % 2, "dec_variant": 0, "mul_window": 4, "dec_window": 6}, bits, path=path)

    ths = [threading.Thread(target=worker, args=(b,)) for b in sizes]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    for b in sizes:
        assert autotune.load(b, path=path)["variant"] == b % 2
