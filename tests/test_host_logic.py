"""Host-side logic without a GPU: the autotuner's choice rule and the
cluster counts the run loop logs at snapshot steps."""
import numpy as np

from gplum_gb300.autotune import keep_incumbent
from gplum_gb300.run import cluster_counts


def test_keep_incumbent_within_tolerance():
    table = {(128, 64, 32, 6): 1.0502, (128, 64, 32, 4): 1.0501, (128, 48, 32, 6): 1.0692}
    best = min(table, key=table.get)
    assert best == (128, 64, 32, 4)
    # within 1 %: the incumbent stays
    assert keep_incumbent(best, table, (128, 64, 32, 6)) == (128, 64, 32, 6)
    # more than 1 % slower: the best measured one wins
    assert keep_incumbent(best, table, (128, 48, 32, 6)) == best
    # no incumbent, or one that was not measured: the best measured one
    assert keep_incumbent(best, table, None) == best
    assert keep_incumbent(best, table, (64, 32, 16, 5)) == best


def test_cluster_counts():
    # five clusters; the one with the largest id_cluster has 3 members
    sizes = np.array([2, 7, 3, 4, 3])
    cids = np.array([10, 4, 99, 50, 3])
    got = cluster_counts(100, sizes, cids)
    assert got == {"n_cluster": 5, "n_isolated": 100 - 19, "largest_cluster": 7,
                   "largest_cluster_as_gplum_logs": 3}
    # no clusters at all
    got = cluster_counts(42, np.zeros(0, np.int64), np.zeros(0, np.int64))
    assert got == {"n_cluster": 0, "n_isolated": 42, "largest_cluster": 0, "largest_cluster_as_gplum_logs": 0}
