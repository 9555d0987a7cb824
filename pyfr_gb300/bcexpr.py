"""Boundary values and source terms given as expressions.

The reference substitutes the options of a ``[soln-bcs-<name>]`` section
(``rho``, ``p``, ``u``, ``v``, ``w``, ``cpTw``) into its boundary kernels as C
expressions of the flux point's coordinates ``x``, ``y``, ``z`` and the time
``t``, with ``[constants]`` substituted (``pyfr/solvers/baseadvec/
inters.py:95-116``), and the options of ``[solver-plugin-source]`` into the
``negdivconf`` kernel as C expressions of ``ploc[i]``, the solution ``u[i]``
and ``t`` (``pyfr/plugins/source.py:15-31``,
``pyfr/plugins/kernels/source.mako``).  Here an expression is compiled
once, on the host, into a short postfix program that the kernels evaluate
per point; a subexpression of constants is folded to a number, so a
constant option costs nothing.  Programs are straight-line (no jumps), and
their stack depth is checked against the kernels' fixed stack.
"""

import ast
import math

import numpy as np

# Opcodes of b200_bcop_t
OPS = {name: i for i, name in enumerate(
    ['const', 'x', 'y', 'z', 't', 'add', 'sub', 'mul', 'div', 'pow', 'neg',
     'sin', 'cos', 'tan', 'exp', 'log', 'sqrt', 'tanh', 'abs', 'asin',
     'acos', 'atan', 'sinh', 'cosh', 'atan2', 'min', 'max', 'floor',
     'ceil', 'u'])}

# Largest stack depth of a program (the kernels' stack size)
MAX_DEPTH = 16

_UNARY = {'sin': math.sin, 'cos': math.cos, 'tan': math.tan,
          'exp': math.exp, 'log': math.log, 'sqrt': math.sqrt,
          'tanh': math.tanh, 'abs': abs, 'fabs': abs, 'asin': math.asin,
          'acos': math.acos, 'atan': math.atan, 'sinh': math.sinh,
          'cosh': math.cosh, 'floor': math.floor, 'ceil': math.ceil}
_BINARY = {'pow': math.pow, 'atan2': math.atan2, 'min': min, 'max': max,
           'fmin': min, 'fmax': max}
_BINOPS = {ast.Add: 'add', ast.Sub: 'sub', ast.Mult: 'mul', ast.Div: 'div',
           ast.Pow: 'pow'}
_PYOP = {'add': lambda a, b: a + b, 'sub': lambda a, b: a - b,
         'mul': lambda a, b: a*b, 'div': lambda a, b: a/b,
         'pow': math.pow}
_VARS = {'x': 0, 'y': 1, 'z': 2}


class BCExpr:
    """A compiled expression: ``const`` (a float) when it depends on
    neither position, time nor solution, otherwise ``prog`` (a list of
    (opcode, value); for ``u`` the value is the variable's index) with
    ``depth`` and the flags ``uses_x``, ``uses_t`` and ``uses_u``.

    Coordinates are written ``x``, ``y``, ``z`` or ``ploc[i]``; solution
    variables (``nvars`` of them, 0 for boundary values) ``u[i]``."""

    def __init__(self, text, ndims, nvars=0):
        self.text = text
        self.ndims = ndims
        self.nvars = nvars
        tree = ast.parse(text.strip(), mode='eval').body
        self.uses_x = self.uses_t = self.uses_u = False
        node = self._fold(tree)
        if isinstance(node, float):
            self.const, self.prog, self.depth = node, [], 1
        else:
            self.const = None
            self.prog = []
            self.depth = self._emit(node)
            if self.depth > MAX_DEPTH:
                raise ValueError(f'Expression {text!r} is too deep for the '
                                 'boundary kernels')

    # The folded tree: floats for constant subtrees, else tuples
    def _fold(self, n):
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)):
            return float(n.value)
        if isinstance(n, ast.Subscript) and isinstance(n.value, ast.Name) \
                and isinstance(n.slice, ast.Constant) and \
                type(n.slice.value) is int:
            a, i = n.value.id, n.slice.value
            if a == 'ploc' and 0 <= i < self.ndims:
                self.uses_x = True
                return ('var', 'xyz'[i])
            if a == 'u' and 0 <= i < self.nvars:
                self.uses_u = True
                return ('u', i)
            raise ValueError(f'{a}[{i}] in {self.text!r}')
        if isinstance(n, ast.Name):
            if n.id in _VARS:
                if _VARS[n.id] >= self.ndims:
                    raise ValueError(f'{n.id} in a {self.ndims}-D boundary '
                                     'expression')
                self.uses_x = True
                return ('var', n.id)
            if n.id == 't':
                self.uses_t = True
                return ('var', 't')
            if n.id == 'pi':
                return math.pi
            raise ValueError(f'Unknown name {n.id!r} in {self.text!r}')
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, (ast.USub,
                                                             ast.UAdd)):
            a = self._fold(n.operand)
            if isinstance(n.op, ast.UAdd):
                return a
            return -a if isinstance(a, float) else ('neg', a)
        if isinstance(n, ast.BinOp) and type(n.op) in _BINOPS:
            op = _BINOPS[type(n.op)]
            a, b = self._fold(n.left), self._fold(n.right)
            if isinstance(a, float) and isinstance(b, float):
                return float(_PYOP[op](a, b))
            return (op, a, b)
        if isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and \
                not n.keywords:
            f, args = n.func.id, [self._fold(a) for a in n.args]
            if f in _UNARY and len(args) == 1:
                name = 'abs' if f == 'fabs' else f
                if isinstance(args[0], float):
                    return float(_UNARY[f](args[0]))
                return (name, args[0])
            if f in _BINARY and len(args) == 2:
                name = {'fmin': 'min', 'fmax': 'max'}.get(f, f)
                if all(isinstance(a, float) for a in args):
                    return float(_BINARY[f](*args))
                return (name, *args)
        raise ValueError(f'Unsupported boundary expression {self.text!r}')

    def _emit(self, node):
        """Append the postfix code of ``node``; returns its stack depth."""
        if isinstance(node, float):
            self.prog.append((OPS['const'], node))
            return 1
        if node[0] == 'var':
            self.prog.append((OPS[node[1]], 0.0))
            return 1
        if node[0] == 'u':
            self.prog.append((OPS['u'], float(node[1])))
            return 1
        op, *args = node
        depths = []
        for i, a in enumerate(args):
            depths.append(i + self._emit(a))
        self.prog.append((OPS[op], 0.0))
        return max(depths)

    def eval_np(self, x, t, u=None):
        """numpy evaluation at the points x (ndims, n), time t and
        solution u (nvars, n) (the same operations, for the host and for
        tests)."""
        if self.const is not None:
            return np.full(x.shape[1], self.const)
        st = []
        for op, v in self.prog:
            name = _NAMES[op]
            if name == 'const':
                st.append(np.full(x.shape[1], v))
            elif name in _VARS:
                st.append(np.asarray(x[_VARS[name]], dtype=float))
            elif name == 'u':
                st.append(np.asarray(u[int(v)], dtype=float))
            elif name == 't':
                st.append(np.full(x.shape[1], float(t)))
            elif name == 'neg':
                st.append(-st.pop())
            elif name in _NPBIN:
                b, a = st.pop(), st.pop()
                st.append(_NPBIN[name](a, b))
            else:
                st.append(_NPUN[name](st.pop()))
        return st[0]


def pack(progs):
    """The programs ``progs`` (lists of (opcode, value)) one after the
    other as an array of ``b200_bcop_t`` (op, pad, val; pad holds the
    variable index of a ``u`` instruction), with each program's start and
    length."""
    ops, spans = [], []
    for p in progs:
        spans.append((len(ops), len(p)))
        ops.extend(p)
    arr = np.zeros(len(ops), dtype=[('op', '<i4'), ('pad', '<i4'),
                                    ('val', '<f8')])
    arr['op'] = [o for o, _ in ops]
    arr['val'] = [v for _, v in ops]
    arr['pad'] = [int(v) if o == OPS['u'] else 0 for o, v in ops]
    return arr, spans


_NAMES = {v: k for k, v in OPS.items()}
_NPBIN = {'add': np.add, 'sub': np.subtract, 'mul': np.multiply,
          'div': np.divide, 'pow': np.power, 'atan2': np.arctan2,
          'min': np.minimum, 'max': np.maximum}
_NPUN = {'sin': np.sin, 'cos': np.cos, 'tan': np.tan, 'exp': np.exp,
         'log': np.log, 'sqrt': np.sqrt, 'tanh': np.tanh, 'abs': np.abs,
         'asin': np.arcsin, 'acos': np.arccos, 'atan': np.arctan,
         'sinh': np.sinh, 'cosh': np.cosh, 'floor': np.floor,
         'ceil': np.ceil}
