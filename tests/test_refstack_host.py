"""PyFR's own host code (its system, interfaces, RK45 integrator and
backend registry, from the reference's source tree) drives the b200
backend: with the library stand-in of ``tests/fake_lib.py`` the whole
construction and a step run on a machine without a GPU, through the
backend interface only.  The numbers are checked on the GPU
(``tests/test_gpu_refstack.py``)."""
import subprocess
import sys

import numpy as np
import pytest

from tests.refstack import ROOT, reference_tree


@pytest.mark.parametrize('case', ['vortex', 'tgv'])
def test_reference_stack_builds_and_steps(tmp_path, case):
    if reference_tree() is None:
        pytest.skip('reference source tree not present')
    out = tmp_path / 'soln.npz'
    r = subprocess.run([sys.executable, '-m', 'tests.refstack', '--fake',
                        '--case', case, '--n', '3', '--steps', '2',
                        '--out', str(out)], cwd=ROOT, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    d = np.load(out)
    assert str(d['backend']) == 'B200Backend'
    assert int(d['nsteps']) == 2
