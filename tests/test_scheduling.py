"""The z-chunk autotuner's search, with a synthetic cost model in place of GPU timing."""

from compiler import scheduling


def test_coordinate_descent_finds_the_best_depth_per_bucket(tmp_path, monkeypatch):
    monkeypatch.setattr(scheduling, "CACHE", tmp_path / "tuned.json")
    shapes = [(64, 64, 32), (128, 96, 64), (256, 256, 96), (64, 128, 96)]
    best = {"nz<=32": 16, "nz<=64": 32, "nz<=96": 48}

    def cost(kz_list):
        return 1.0 + sum(abs(k - best[scheduling.bucket(nz)]) for k, (_, _, nz) in zip(kz_list, shapes)) / 100.0

    result = scheduling.tune(shapes, "TestGPU", 1, cost)
    assert result["choice"] == best
    assert scheduling.kz_for(shapes, "TestGPU", 1) == [16, 32, 48, 48]
    assert scheduling.kz_for(shapes, "OtherGPU", 1) == [scheduling.DEFAULT_KZ] * 4


def test_buckets():
    assert scheduling.bucket(32) == "nz<=32" and scheduling.bucket(33) == "nz<=48"
    assert scheduling.bucket(96) == "nz<=96" and scheduling.bucket(1000) == "nz>256"
