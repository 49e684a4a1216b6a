"""The autotuner's JSON cache on the host: save / load per device name and key
size, replace-whole writes, and a damaged file read as empty."""

from heu_gb300 import autotune


def test_save_and_load_round_trip(tmp_path):
    path = str(tmp_path / "sub" / "tuning.json")
    cfg = {"variant": 1, "dec_variant": 0, "mul_window": 4, "dec_window": 6}
    autotune.save(cfg, 2048, path=path, rates={"encrypt": 1.0})
    autotune.save(dict(cfg, variant=0), 3072, path=path)
    assert autotune.load(2048, path=path) == cfg
    assert autotune.load(3072, path=path)["variant"] == 0
    assert autotune.load(1024, path=path) is None
    assert [p.name for p in (tmp_path / "sub").iterdir()] == ["tuning.json"]  # no temporary left behind
    (tmp_path / "sub" / "tuning.json").write_text("{not json")
    assert autotune.load(2048, path=path) is None
    autotune.save(cfg, 2048, path=path)
    assert autotune.load(2048, path=path) == cfg
