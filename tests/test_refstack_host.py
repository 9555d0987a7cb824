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


@pytest.mark.parametrize('source', [False, True])
@pytest.mark.parametrize('case', ['vortex', 'tgv'])
def test_reference_stack_builds_and_steps(tmp_path, case, source):
    """With ``source`` PyFR's own source plugin adds its macro to the
    elements (pyfr/plugins/source.py:26-31) and the b200 backend builds
    negdivconf, copy_soln and evalsrcmacros from it."""
    if reference_tree() is None:
        pytest.skip('reference source tree not present')
    out = tmp_path / 'soln.npz'
    r = subprocess.run([sys.executable, '-m', 'tests.refstack', '--fake',
                        '--case', case, '--n', '3', '--steps', '2',
                        '--out', str(out)] + (['--source'] if source else []),
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    d = np.load(out)
    assert str(d['backend']) == 'B200Backend'
    assert int(d['nsteps']) == 2


def test_reference_divergence_chain_fused(tmp_path):
    """With fused operator applies, the fuser turns the divergence chain
    PyFR's Euler system groups (tdivtpcorf, tdivtconf, negdivconf;
    pyfr/solvers/baseadvec/system.py:126-132) into one tensor-core apply."""
    import json
    if reference_tree() is None:
        pytest.skip('reference source tree not present')
    r = subprocess.run([sys.executable, '-m', 'tests.refstack', '--fake',
                        '--case', 'vortex', '--n', '3', '--steps', '1',
                        '--single', '--report'], cwd=ROOT,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    graphs = json.loads(r.stdout.strip().splitlines()[-1])
    names = [n for g in graphs for n in g]
    assert 'mul:bf16x3-cat' in names
    assert 'negdivconf' not in names
    assert graphs[-1] == ['tflux', 'mul:bf16x3-cat']


@pytest.mark.parametrize('kinds', ['hex-pyr-tet', 'pri-tet'])
def test_reference_stack_mixed_mesh_builds_and_steps(tmp_path, kinds):
    """PyFR's own Euler system on a mixed mesh (its own pyramid shape and
    points with hexahedra and tetrahedra, or prisms with tetrahedra) builds
    every kernel it asks for from the b200 backend and steps, against the
    library stand-in (no GPU)."""
    if reference_tree() is None:
        pytest.skip('reference source tree not present')
    out = tmp_path / 'soln.npz'
    r = subprocess.run([sys.executable, '-m', 'tests.refstack', '--fake',
                        '--case', f'mixed-{kinds}', '--n', '2', '--steps',
                        '2', '--out', str(out)],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    d = np.load(out)
    assert str(d['backend']) == 'B200Backend'
    assert int(d['nsteps']) == 2
    assert set(map(str, d['etypes'])) == set(kinds.split('-'))
