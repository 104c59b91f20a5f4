"""The autotuner's host logic and the committed table it produced (no GPU):
the table holds only launch variants that keep a size's arithmetic, the
split-exchange form only where a size has 32 values per thread, and the
choice rules (1 % over the plain kernel; a change of values per thread
resets that size's launch variants) hold on synthetic measurements."""
import os
import re

from conftest import ROOT

from ckfft_gb300 import autotune as at

TABLE = os.path.join(ROOT, "ckfft_gb300", "csrc", "tuning_table.h")


def parse_table(path):
    text = open(path).read()
    lr = [int(v) for v in re.search(r"kTunedLog2R\[\d+\]\s*=\s*\{([0-9, ]+)\}", text).group(1).split(",")]
    rows = re.findall(r"\{([0-9, ]+)\},\s*//\s*(\w+)", text)
    return lr, {kind: [int(v) for v in row.split(",")] for row, kind in rows}


def test_committed_table_is_well_formed():
    lr, table = parse_table(TABLE)
    assert len(lr) == len(at.LOG2_RANGE)
    assert sorted(table) == sorted(at.KINDS)
    for kind, row in table.items():
        assert len(row) == len(at.LOG2_RANGE), kind
        for L, v in enumerate(row):
            # launch variants only: the values per thread live in kTunedLog2R
            assert v == 0 or v in at.SAME_BITS, (kind, L, v)
            # the split-exchange form exists for 32 values per thread only
            if v == 8:
                assert lr[L] == 5, (kind, L)
    # values per thread never exceed the size (radix <= length)
    for L, r in enumerate(lr):
        assert 0 <= r <= max(L, 0) or (L == 0 and r == 0), (L, r)


def synthetic(plain=100.0, overrides=None):
    """results[variant][kind][str(L)] = GB/s; every variant equal to plain
    unless overridden by {(variant, kind, L): gbs}."""
    res = {v: {k: {str(L): plain for L in at.LOG2_RANGE} for k in at.KINDS} for v in at.VARIANTS}
    for (v, k, L), g in (overrides or {}).items():
        res[v][k][str(L)] = g
    return res


def test_choose_takes_a_launch_variant_only_above_one_percent():
    lr0 = at.current_log2r()
    res = synthetic(overrides={(7, "cfwd", 10): 100.5, (8, "cinv", 14): 102.0, (2, "rinv", 11): 103.0,
                               (3, "rinv", 11): 104.0})
    lr, table = at.choose(res, lr0)
    assert lr == lr0
    ki = {k: i for i, k in enumerate(at.KINDS)}
    assert table[ki["cfwd"]][10] == 0          # 0.5 % is noise
    assert table[ki["cinv"]][14] == 8
    assert table[ki["rinv"]][11] == 3          # the best of the qualifying variants
    assert sum(v != 0 for row in table for v in row) == 2


def test_choose_changes_values_per_thread_and_resets_launch_variants():
    lr0 = at.current_log2r()
    L = 9
    # half the values per thread wins summed over the four kinds by > 1 %;
    # a launch variant measured with the old values per thread is dropped
    over = {(4, k, L): 103.0 for k in at.KINDS}
    over[(7, "cfwd", L)] = 110.0
    lr, table = at.choose(synthetic(overrides=over), lr0)
    assert lr[L] == lr0[L] - 1
    assert all(table[i][L] == 0 for i in range(len(at.KINDS)))
    # twice the values per thread loses: nothing changes
    lr2, _ = at.choose(synthetic(overrides={(5, k, L): 99.0 for k in at.KINDS}), lr0)
    assert lr2 == lr0


def test_write_outputs_round_trips_through_the_table_parser(tmp_path):
    res = synthetic(overrides={(8, "cfwd", 14): 120.0})
    at.write_outputs(res, str(tmp_path), "test GPU")
    lr, table = parse_table(os.path.join(tmp_path, "tuning_table.h"))
    assert lr == at.current_log2r()
    assert table["cfwd"][14] == 8
    md = open(os.path.join(tmp_path, "autotune.md")).read()
    assert "| cfwd | 14 |" in md and "pipe sx" in md
