"""Boundary-value expressions compiled to postfix programs (CPU): constant
folding, evaluation against numpy's evaluation of the same text, stack
depth, and the errors."""
import numpy as np
import pytest

from pyfr_gb300.bcexpr import MAX_DEPTH, OPS, BCExpr

NP = dict(sin=np.sin, cos=np.cos, tan=np.tan, exp=np.exp, log=np.log,
          sqrt=np.sqrt, tanh=np.tanh, fabs=np.abs, abs=np.abs,
          atan2=np.arctan2, pow=np.power, fmin=np.minimum, fmax=np.maximum,
          pi=np.pi)

EXPRS = ['1.5', '2*pi/3 + sqrt(2)', '1 + 0.1*sin(2*pi*x - t)',
         'pow(1 + 0.2*y, 1.4) - fabs(x)', '-x*y + exp(-t)*cos(3*y)',
         'fmax(0.1, tanh(5*(x - 0.5))) + atan2(y, 1 + x*x)',
         '(x - 0.5)**2 + (y - 0.5)**2', 'log(2 + x)/(1 + t*t)']


@pytest.mark.parametrize('text', EXPRS)
def test_eval_matches_numpy(text):
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, (2, 50))
    t = 0.37
    ex = BCExpr(text, 2)
    ref = eval(text, {'__builtins__': {}},
               NP | dict(x=x[0], y=x[1], t=t))
    np.testing.assert_allclose(ex.eval_np(x, t),
                               np.broadcast_to(ref, (50,)), rtol=1e-14,
                               atol=1e-14)
    import re
    if not re.search(r'\b[xyt]\b', text):
        assert ex.const is not None and ex.prog == []
    else:
        assert ex.const is None and 1 <= ex.depth <= MAX_DEPTH


def test_folding_and_flags():
    ex = BCExpr('2*3 + x*(4 - 1)', 2)
    # 6 + x*3: const 6, x, const 3, mul, add
    assert [op for op, _ in ex.prog] == [OPS['const'], OPS['x'], OPS['const'],
                                         OPS['mul'], OPS['add']]
    assert ex.uses_x and not ex.uses_t and ex.depth == 3
    assert BCExpr('sin(t)', 3).uses_t


@pytest.mark.parametrize('text,nd', [('q + 1', 2), ('z', 2), ('x if t else y', 2),
                                     ('foo(x)', 3)])
def test_errors(text, nd):
    with pytest.raises(ValueError):
        BCExpr(text, nd)


def test_depth_limit():
    deep = 'x'
    for _ in range(MAX_DEPTH + 2):
        deep = f'x*({deep} + 1)'
    # x*(x*(... + 1) + 1): each level keeps one more value on the stack
    with pytest.raises(ValueError):
        BCExpr(deep, 2)
