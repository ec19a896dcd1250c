"""Planner wisdom: the planner measurement's kernel choices exported to and
imported from a text file (the counterpart of FFTW's wisdom, which the
reference's FFTW planner accumulates under fftw_flags = FFTW.MEASURE and
FFTW.jl exports / imports).  The file handling needs no GPU; the GPU test
checks that a measured plan's choices are reused after a forget / import
cycle and that the results stay those of the oracle."""
import numpy as np
import pytest

import pencilffts_gb300 as P


def test_wisdom_file_round_trip(tmp_path):
    P.forget_wisdom()
    assert P.wisdom_stats() == (0, 0)
    f = tmp_path / "empty.wisdom"
    P.export_wisdom(f)
    assert f.read_text().splitlines() == ["pencilfft_gb300 wisdom 1"]
    g = tmp_path / "two.wisdom"
    g.write_text("pencilfft_gb300 wisdom 1\n1\tc2r-tma|devA|rb8|pr0|op2|s1|M512|x\n"
                 "2\tbluestein-generic|devA|rb4|pr0|op0|s-1|M97|y\n")
    P.import_wisdom(g)
    assert P.wisdom_stats()[0] == 2
    h = tmp_path / "out.wisdom"
    P.export_wisdom(h)
    assert sorted(h.read_text().splitlines()[1:]) == sorted(g.read_text().splitlines()[1:])
    P.forget_wisdom()
    assert P.wisdom_stats() == (0, 0)


@pytest.mark.parametrize("text", ["something else\n", "pencilfft_gb300 wisdom 1\nx\tkey\n",
                                  "pencilfft_gb300 wisdom 1\n7\tkey\n", "pencilfft_gb300 wisdom 1\n1\t\n"])
def test_wisdom_rejects_other_files(tmp_path, text):
    f = tmp_path / "bad.wisdom"
    f.write_text(text)
    with pytest.raises(P.ArgumentError):
        P.import_wisdom(f)
    with pytest.raises(P.ArgumentError):
        P.import_wisdom(tmp_path / "missing.wisdom")


@pytest.mark.gpu
def test_wisdom_reused_by_measured_plans(cuda, tmp_path):
    from helpers import T
    from test_gpu_parity import check_plan
    P.forget_wisdom()
    dims = (97, 64, 40)  # Bluestein lines along x, measured in both directions
    plan = P.PencilFFTPlan(dims, T.RFFT(), np.float32, fftw_flags=P.FFTW_MEASURE)
    entries, hits = P.wisdom_stats()
    assert entries >= 2 and hits == 0  # the x pass in both directions was measured
    f = tmp_path / "w.wisdom"
    P.export_wisdom(f)
    P.forget_wisdom()
    P.import_wisdom(f)
    plan2 = P.PencilFFTPlan(dims, T.RFFT(), np.float32, fftw_flags=P.FFTW_MEASURE)
    assert P.wisdom_stats() == (entries, entries)  # every measured pass answered by the file
    check_plan(plan2, seed=3)
    check_plan(plan, seed=3)
    P.forget_wisdom()
