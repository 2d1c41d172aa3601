"""The autotuner's selection rule and the committed table, on the CPU.

The GPU measurement itself runs on a GB300 (python -m vkhel_gb300.autotune);
what it keeps from a measurement is host logic: per (degree, jobs-per-SM
bucket) the fastest variant, unless the incumbent -- variant 0 for the
many-jobs bucket, the many-jobs choice for the others -- is within 2 % of
it.  The committed table must be what that rule makes of the committed
report, and name a variant for every degree, bucket and family.
"""
import json
import os

from conftest import ROOT
from vkhel_gb300 import autotune

TUNING = os.path.join(ROOT, "vkhel_gb300", "tuning")


def test_choose_keeps_the_incumbent_within_the_margin():
    assert autotune.choose({0: 1.00, 1: 0.99}, 0) == 0       # 1 % faster: noise
    assert autotune.choose({0: 1.00, 1: 0.97}, 0) == 1       # 3 % faster: taken
    assert autotune.choose({0: 1.00, 1: 0.97, 2: 0.98}, 2) == 2
    assert autotune.choose({0: 1.00, 2: 0.90}, 1) == 2       # incumbent not measured here


def test_committed_table_follows_from_the_committed_report():
    report = json.load(open(os.path.join(TUNING, "gb300_report.json")))
    want = autotune.table_from_report(report)
    got = {}
    for line in open(os.path.join(TUNING, "gb300.txt")):
        f = line.split("#")[0].split()
        if len(f) == 4:
            got[(int(f[0]), int(f[1]), int(f[3]))] = int(f[2])
    assert got == want
    for fam in (0, 1, 2):
        for log_n in range(8, 15):
            for bucket in range(4):
                assert (fam, log_n, bucket) in got
    assert report["batch_classes"]["chosen"] in ("sequential", "concurrent", "single_launch")
