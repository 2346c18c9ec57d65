"""GPU: the profiling driver (python -m gpucadforam_gb300.kernel_cases) runs
each of its cases, the commands the ncu summaries cite."""
import json

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["unit_cell", "lattice_rows", "lattice_wide", "lattice_params", "lattice_blend",
                                  "staged_mc"])
def test_kernel_case_runs(case, capsys):
    from gpucadforam_gb300 import kernel_cases

    assert kernel_cases.main([case, "--n", "48", "--reps", "1"]) == 0
    info = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert info["case"] == case and info["grid"] == 48 and info["ms"] > 0
    if case == "staged_mc":
        assert info["verts"] > 0 and info["verts"] % 3 == 0
