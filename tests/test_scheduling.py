"""The batched-step autotuner's search, with a synthetic cost model in place of GPU timing."""

from compiler import scheduling


def test_coordinate_descent_finds_the_best_depth_per_bucket(tmp_path, monkeypatch):
    monkeypatch.setattr(scheduling, "CACHE", tmp_path / "tuned.json")
    shapes = [(64, 64, 32), (128, 96, 64), (256, 256, 96), (64, 128, 96)]
    best = {"nz<=32": 16, "nz<=64": 32, "nz<=96": 48}
    seen_rows = set()

    def cost(kz_list, rows):
        seen_rows.add(rows)
        return 1.0 + sum(abs(k - best[scheduling.bucket(nz)]) for k, (_, _, nz) in zip(kz_list, shapes)) / 100.0

    result = scheduling.tune(shapes, "TestGPU", 1, cost)
    assert result["choice"] == {**best, "tile_rows": 8}
    assert seen_rows == {8}  # the strict kernel has 8-row tiles only
    assert scheduling.kz_for(shapes, "TestGPU", 1) == [16, 32, 48, 48]
    assert scheduling.kz_for(shapes, "OtherGPU", 1) == [scheduling.DEFAULT_KZ] * 4
    assert scheduling.rows_for("TestGPU", 1) == 8


def test_fast_fp_tuning_picks_a_tile_height_and_depths(tmp_path, monkeypatch):
    monkeypatch.setattr(scheduling, "CACHE", tmp_path / "tuned.json")
    shapes = [(64, 64, 32), (96, 64, 32), (256, 256, 96)]
    best = {"nz<=32": 8, "nz<=96": 24}

    def cost(kz_list, rows):
        # 16-row tiles are best, whatever the depths; the depths add their own penalty
        depth = sum(abs(k - best[scheduling.bucket(nz)]) for k, (_, _, nz) in zip(kz_list, shapes))
        return {4: 1.3, 8: 1.1, 16: 1.0}[rows] + depth / 100.0

    result = scheduling.tune(shapes, "TestGPU", 1, cost, numerics="fast")
    assert result["choice"] == {**best, "tile_rows": 16}
    assert scheduling.rows_for("TestGPU", 1, numerics="fast") == 16
    assert scheduling.kz_for(shapes, "TestGPU", 1, numerics="fast") == [8, 8, 24]
    # the strict contract keeps its own table (untuned here): 8 rows and the default depth
    assert scheduling.rows_for("TestGPU", 1) == 8
    assert scheduling.kz_for(shapes, "TestGPU", 1) == [scheduling.DEFAULT_KZ] * 3


def test_buckets():
    assert scheduling.bucket(32) == "nz<=32" and scheduling.bucket(33) == "nz<=48"
    assert scheduling.bucket(96) == "nz<=96" and scheduling.bucket(1000) == "nz>256"
