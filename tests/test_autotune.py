"""CPU test of the autotuner's search (atag.autotune.coordinate_descent)."""
from atag import autotune


def test_coordinate_descent_finds_separable_optimum():
    target = {"ccl_tile_rows": 8, "boundary_tile_rows": 16, "small_cluster_max": 2048,
              "small_ctas_per_sm": 12, "large_ctas_divisor": 1, "index_ctas_per_sm": 16, "batch_lanes": 2}
    calls = []

    def cost(t):
        calls.append(dict(t))
        return sum(abs(autotune.SPACE[k].index(t[k]) - autotune.SPACE[k].index(target[k])) for k in t) + 1.0

    start = {"ccl_tile_rows": 16, "boundary_tile_rows": 16, "small_cluster_max": 512,
             "small_ctas_per_sm": 4, "large_ctas_divisor": 4, "index_ctas_per_sm": 8, "batch_lanes": 1}
    best, ms, log = autotune.coordinate_descent(cost, start)
    assert best == target and ms == 1.0
    assert len(calls) == len(log) < 40


def test_coordinate_descent_keeps_start_when_nothing_is_faster():
    start = {k: v[0] for k, v in autotune.SPACE.items()}
    best, ms, log = autotune.coordinate_descent(lambda t: 5.0, start, passes=3)
    assert best == start and ms == 5.0
