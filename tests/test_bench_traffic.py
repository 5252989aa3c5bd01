"""bench.py's roofline `traffic`: the DRAM bytes per launch of the reported smoother kernel, read from the committed
ncu summaries in profiles/ (one column per captured launch) and weighted by the bench's own launches (CPU only)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_profile_columns_parse():
    import bench
    cols = bench.profiled_columns("k_rbgs4s_f16_split_finest_pool_sphere_256.md")
    assert len(cols) == 2  # a pressure launch and a potential launch
    for traffic, alg in cols:
        assert 10.0 < traffic < 1000.0 and 10.0 < alg < 1000.0
    assert bench.profiled_columns("k_rbgs4_f16_finest_pool_sphere_256.md")[0][0] > 0
    assert bench.profiled_columns("no_such_summary.md") == []
    assert bench.profiled_columns(None) == []


def test_traffic_weighted_by_the_bench_launches():
    import bench
    cols = bench.profiled_columns("k_rbgs4s_f16_split_finest_pool_sphere_256.md")
    # launches at the capture's own algorithmic bytes reproduce the capture's traffic, weighted by launch counts
    per_solve = [(3, cols[0][1] * 1e6), (1, cols[1][1] * 1e6)]
    t = bench.profiled_traffic("k_rbgs4s_f16_split_finest_pool_sphere_256.md", 256, per_solve)
    assert abs(t - 1e6 * (3 * cols[0][0] + cols[1][0]) / 4) <= 1
    # twice the algorithmic bytes (a larger grid) doubles the traffic
    t2 = bench.profiled_traffic("k_rbgs4s_f16_split_finest_pool_sphere_256.md", 256,
                                [(k, 2 * b) for k, b in per_solve])
    assert abs(t2 - 2 * t) <= 2
    # a single-column capture scales with the cell count
    t3 = bench.profiled_traffic("k_rbgs4_f16_finest_pool_sphere_256.md", 128)
    assert abs(t3 - 1e6 * bench.profiled_columns("k_rbgs4_f16_finest_pool_sphere_256.md")[0][0] / 8) <= 1
