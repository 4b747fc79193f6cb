"""The artifact's result tables (compiled/run.sh, run_sconf.sh) from this engine."""
import csv

import numpy as np
import pytest

from gbstencil import capi, report


def test_max_degree_matches_plan():
    # 3-D radius >= 3 kernels are built for one fused step only; 2-D stars to 8
    # (FMA); 3-D FMA tiles to 8 while they keep output rows, exact mode to 2-4
    assert report.max_degree("star3d3r", np.float32, "fma") == 1
    assert report.max_degree("star2d1r", np.float32, "fma") == 8
    assert report.max_degree("j3d27pt", np.float64, "fma") == 8
    assert report.max_degree("star3d2r", np.float32, "fma") == 4
    assert report.max_degree("j3d27pt", np.float64, "exact") == 2
    assert report.max_degree("box3d1r", np.float32, "exact") == 4


@pytest.mark.gpu
def test_sweep_csv(tmp_path):
    report.main(["sweep", "--out", str(tmp_path), "-t", "4", "-n", "1", "--s3", "48", "--stencils", "star3d2r",
                 "--bt-max", "2"])
    rows = list(csv.reader(open(tmp_path / "sweep.csv")))
    assert rows[0][:3] == ["Stencil", "Precision", "bT"]
    assert [(r[1], r[2]) for r in rows[1:]] == [("float", "1"), ("float", "2"), ("double", "1"), ("double", "2")]
    assert all(float(r[8]) > 0 for r in rows[1:])


def test_sconf_stencils_are_the_papers_seven():
    assert report.SCONF_STENCILS == ["j2d5pt", "j2d9pt-gol", "j2d9pt", "gradient2d", "star3d1r", "star3d2r", "j3d27pt"]
    assert all(n in capi.NAMES for n in report.SCONF_STENCILS)


@pytest.mark.gpu
def test_run_csv_format(tmp_path):
    report.main(["run", "--prec", "float", "--out", str(tmp_path), "-t", "4", "-n", "1", "--s2", "256",
                 "--s3", "48", "--stencils", "star2d1r,j3d27pt"])
    rows = list(csv.reader(open(tmp_path / "float_run.csv")))
    assert rows[0] == ["Stencil", "bS1", "bS2", "bT", "sl", "Model", "Measured"]
    assert [r[0] for r in rows[1:]] == ["star2d1r", "j3d27pt"]
    two, three = rows[1], rows[2]
    assert two[2] == "" and three[2] != ""          # bS2 only for 3-D, as run.sh writes it
    for r in rows[1:]:
        assert int(r[3]) >= 1 and float(r[6]) > 0 and float(r[5].replace(",", "")) > 0


@pytest.mark.gpu
def test_sconf_csv(tmp_path):
    report.main(["sconf", "--out", str(tmp_path), "-t", "8", "-n", "1", "--s2", "256", "--s3", "48"])
    rows = list(csv.reader(open(tmp_path / "sconf.csv")))
    assert len(rows) == 1 + 2 * len(report.SCONF_STENCILS)
    for r in rows[1:]:
        assert int(r[4]) <= 4 and float(r[6]) > 0
