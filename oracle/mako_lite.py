"""A renderer for the part of the Mako template language that the
reference's kernel templates use.  Test infrastructure only: it renders the
reference's own ``.mako`` kernel sources into C so that the reference's
pointwise arithmetic can be compiled with gcc and evaluated on the host
(``oracle/refkernels.py``).  Nothing in the product imports it.

Mako itself (``mako>=1.0``, pyproject.toml:27 of the reference) is not
installed.  The constructs handled are the ones the kernel templates under
``pyfr/solvers``, ``pyfr/integrators`` and ``pyfr/backends/*/kernels`` use:

* text with ``${expr}`` substitutions (``str`` of the value);
* control lines ``% for``/``% if``/``% elif``/``% else``/``% endfor``/
  ``% endif`` (and ``% while``), and ``##`` comment lines;
* ``<% code %>`` blocks;
* ``<%namespace module='m' name='n'/>``: ``n.f(*a)`` calls ``m.f(context,
  *a)`` (Mako's module namespaces);
* ``<%include file='...'/>`` and ``<%inherit file='...'/>`` (with
  ``${next.body()}`` in the parent), file names may hold ``${...}``;
* call tags ``<%n:f a='..'>body</%n:f>`` and self-closing ``<%n:f a='..'/>``:
  the body becomes ``caller.body`` (with the signature given by an ``args``
  attribute), attribute values are strings with ``${...}`` interpolated;
* the runtime helpers ``capture`` and ``supports_caller`` of
  ``mako.runtime`` (installed as a module ``mako.runtime`` by
  ``install_runtime``, so that the reference's ``makoutil`` imports).

Templates are found by dotted name the way the reference's
``pyfr/template.py:DottedTemplateLookup`` finds them (package path + name +
``.mako``), with source filters applied before parsing, and any name may be
overridden by a literal source (used for the backend ``base`` template,
which is this package's own).
"""

import os
import re
import sys
import types


class Context:
    """Template variables plus the output buffer stack and the stack of
    call-tag callers (``context['caller']``)."""

    def __init__(self, data, lookup):
        self._data = dict(data)
        self._bufs = [[]]
        self._callers = [None]
        self.lookup = lookup

    def __getitem__(self, k):
        if k == 'caller':
            return self._callers[-1]
        return self._data[k]

    def __contains__(self, k):
        return k in self._data

    def get(self, k, default=None):
        return self._data.get(k, default)

    def keys(self):
        return self._data.keys()

    def write(self, s):
        self._bufs[-1].append(s)

    def push_buffer(self):
        self._bufs.append([])

    def pop_buffer(self):
        return ''.join(self._bufs.pop())


def capture(context, fn, *args, **kwargs):
    """Run ``fn`` with its output redirected; return that output."""
    context.push_buffer()
    try:
        fn(*args, **kwargs)
    finally:
        out = context.pop_buffer()
    return out


def supports_caller(fn):
    """The caller of a call tag is pushed by the tag itself before the
    call, so the decorated function only needs the context passed on."""
    def wrapped(context, *args, **kwargs):
        return fn(context, *args, **kwargs)
    wrapped.__name__ = fn.__name__
    wrapped.__wrapped__ = fn
    return wrapped


def install_runtime():
    """Make ``import mako.runtime`` resolve to this module's helpers."""
    if 'mako.runtime' in sys.modules and \
            getattr(sys.modules['mako.runtime'], '_lite', False):
        return
    pkg = types.ModuleType('mako')
    pkg.__path__ = []
    rt = types.ModuleType('mako.runtime')
    rt.capture = capture
    rt.supports_caller = supports_caller
    rt._lite = True
    pkg.runtime = rt
    sys.modules['mako'] = pkg
    sys.modules['mako.runtime'] = rt


# ---------------------------------------------------------------------------
# Lexer
# ---------------------------------------------------------------------------

def _match_braces(src, i):
    """Index just past the ``}`` closing the ``{`` at ``src[i]``, skipping
    Python string literals (f-strings' braces included)."""
    depth, n = 0, len(src)
    while i < n:
        ch = src[i]
        if ch in '\'"':
            q = src[i:i + 3] if src[i:i + 3] in ('"""', "'''") else ch
            j = i + len(q)
            while j < n:
                if src[j] == '\\':
                    j += 2
                    continue
                if src.startswith(q, j):
                    break
                j += 1
            i = j + len(q)
            continue
        if ch in '{([':
            depth += 1
        elif ch in '})]':
            depth -= 1
            if depth == 0:
                return i + 1
        i += 1
    raise SyntaxError('Unterminated ${...} expression')


def _tag_end(src, i):
    """Index just past the ``>`` ending the tag opened at ``src[i]``; quoted
    attribute values may hold ``>``."""
    n, q = len(src), None
    while i < n:
        ch = src[i]
        if q:
            if ch == q:
                q = None
        elif ch in '\'"':
            q = ch
        elif ch == '>':
            return i + 1
        i += 1
    raise SyntaxError('Unterminated tag')


_ATTR = re.compile(r'''([\w:]+)\s*=\s*(?:"([^"]*)"|'([^']*)')''', re.S)


def _attrs(text):
    return {m[1]: m[2] if m[2] is not None else m[3]
            for m in _ATTR.finditer(text)}


def lex(src):
    """Token list: ('text', s), ('expr', s), ('control', s), ('code', s),
    ('tag', kind, attrs, selfclosing), ('endtag', kind)."""
    toks, text = [], []
    i, n = 0, len(src)

    def flush():
        if text:
            toks.append(('text', ''.join(text)))
            text.clear()

    while i < n:
        if i == 0 or src[i - 1] == '\n':
            m = re.compile(r'[ \t]*(%|##)(?!%)([^\n]*)(\n|$)').match(src, i)
            if m:
                flush()
                if m[1] == '%':
                    toks.append(('control', m[2].strip()))
                i = m.end()
                continue
        if src.startswith('${', i):
            flush()
            j = _match_braces(src, i + 1)
            toks.append(('expr', src[i + 2:j - 1]))
            i = j
        elif src.startswith('<%!', i) or re.match(r'<%\s', src[i:i + 3]):
            flush()
            j = src.index('%>', i)
            toks.append(('code', src[i + (3 if src[i + 2] == '!' else 2):j]))
            i = j + 2
        elif src.startswith('<%', i) and re.match(r'<%[\w:]', src[i:i + 3]):
            flush()
            j = _tag_end(src, i)
            body = src[i + 2:j - 1]
            selfc = body.endswith('/')
            if selfc:
                body = body[:-1]
            kind = re.match(r'[\w:]+', body)[0]
            toks.append(('tag', kind, _attrs(body[len(kind):]), selfc))
            i = j
        elif src.startswith('</%', i):
            flush()
            j = src.index('>', i)
            toks.append(('endtag', src[i + 3:j].strip()))
            i = j + 1
        elif src.startswith('\\\n', i):
            i += 2
        else:
            text.append(src[i])
            i += 1
    flush()
    return toks


# ---------------------------------------------------------------------------
# Code generation
# ---------------------------------------------------------------------------

def _interp(value):
    """Python expression for an attribute string with ${...} parts."""
    parts, i = [], 0
    while True:
        j = value.find('${', i)
        if j < 0:
            parts.append(repr(value[i:]))
            break
        parts.append(repr(value[i:j]))
        k = _match_braces(value, j + 1)
        parts.append(f'str({value[j + 2:k - 1]})')
        i = k
    return ' + '.join(p for p in parts if p != "''") or "''"


class _Gen:
    def __init__(self):
        self.lines = []
        self.ind = 1
        self.nfn = 0
        self.stack = []          # open control / call blocks

    def emit(self, s):
        self.lines.append('    '*self.ind + s)

    def code_block(self, code):
        lines = code.split('\n')
        # Normalise indentation as Mako does for <% %> blocks
        body = [l for l in lines if l.strip()]
        if not body:
            return
        pad = min(len(l) - len(l.lstrip()) for l in body)
        for l in lines:
            if l.strip():
                self.emit(l[pad:].rstrip())

    def control(self, c):
        kw = re.match(r'\w+', c)[0]
        if kw in ('endfor', 'endif', 'endwhile'):
            if not self.stack or self.stack[-1] != 'ctl':
                raise SyntaxError(f'Unbalanced % {kw}')
            self.stack.pop()
            self.emit('pass')
            self.ind -= 1
        elif kw in ('elif', 'else'):
            self.emit('pass')
            self.ind -= 1
            self.emit(c if c.endswith(':') else c + ':')
            self.ind += 1
        elif kw in ('for', 'if', 'while'):
            self.emit(c if c.endswith(':') else c + ':')
            self.ind += 1
            self.stack.append('ctl')
        else:
            raise SyntaxError(f'Unsupported control line: % {c}')


def compile_template(src):
    """Python source of ``render(context, __w, __next)`` plus the template's
    inherit target (or None)."""
    toks = lex(src)
    g = _Gen()
    inherit = None
    hoisted = []

    # Namespace and inherit tags act before the body (as in Mako)
    for t in toks:
        if t[0] == 'tag' and t[1] == 'namespace':
            a = t[2]
            if 'module' not in a:
                raise NotImplementedError('Only module namespaces')
            hoisted.append(f"{a['name']} = __ns({a['module']!r})")
        elif t[0] == 'tag' and t[1] == 'inherit':
            inherit = t[2]['file']

    for h in hoisted:
        g.emit(h)

    calls = []
    for t in toks:
        kind = t[0]
        if kind == 'text':
            g.emit(f'__w({t[1]!r})')
        elif kind == 'expr':
            g.emit(f'__w(str({t[1].strip()}))')
        elif kind == 'control':
            g.control(t[1])
        elif kind == 'code':
            g.code_block(t[1])
        elif kind == 'tag':
            _, name, attrs, selfc = t
            if name in ('namespace', 'inherit'):
                continue
            elif name == 'include':
                g.emit(f"__include({_interp(attrs['file'])})")
            elif name == 'def':
                raise NotImplementedError('<%def> is not supported')
            elif ':' in name:
                ns, fn = name.split(':', 1)
                args = attrs.pop('args', '')
                kw = ', '.join(f'{k}={_interp(v)}' for k, v in attrs.items())
                g.nfn += 1
                body = f'__body{g.nfn}'
                g.emit(f'def {body}({args}):')
                g.ind += 1
                if selfc:
                    g.emit('pass')
                    g.ind -= 1
                    g.emit(f'__w(str(__call({body}, {ns}.{fn}, {kw})))'
                           if kw else
                           f'__w(str(__call({body}, {ns}.{fn})))')
                else:
                    g.emit('pass')
                    g.stack.append('call')
                    calls.append((name, body, ns, fn, kw))
            else:
                raise NotImplementedError(f'<%{name}> is not supported')
        elif kind == 'endtag':
            name = t[1]
            if not calls or calls[-1][0] != name or g.stack[-1] != 'call':
                raise SyntaxError(f'Unbalanced </%{name}>')
            g.stack.pop()
            _, body, ns, fn, kw = calls.pop()
            g.ind -= 1
            call = f'__call({body}, {ns}.{fn}' + (f', {kw})' if kw else ')')
            g.emit(f'__w(str({call}))')
    if g.stack:
        raise SyntaxError('Unclosed block at end of template')

    src = 'def render(__w, __include, __call, __ns, next):\n'
    src += '\n'.join(g.lines) + '\n    return ""\n'
    return src, inherit


class _ModuleNS:
    def __init__(self, module, context):
        self._m = module
        self._ctx = context

    def __getattr__(self, name):
        fn = getattr(self._m, name)
        ctx = self._ctx
        return lambda *a, **kw: fn(ctx, *a, **kw)


class _Caller:
    def __init__(self, body):
        self.body = body


class _Next:
    def __init__(self, fn):
        self._fn = fn

    def body(self):
        self._fn()
        return ''


class Lookup:
    """Dotted-name template lookup over a source tree (``root`` holds the
    top-level package, e.g. the reference's checkout), with literal
    overrides and source filters."""

    def __init__(self, root, dfltpkg, overrides=None, filters=()):
        self.root = root
        self.dfltpkg = dfltpkg
        self.overrides = dict(overrides or {})
        self.filters = list(filters)
        self._cache = {}

    def source(self, name):
        if name in self.overrides:
            return self.overrides[name]
        div = name.rfind('.')
        pkg, base = (name[:div], name[div + 1:]) if div >= 0 else \
            (self.dfltpkg, name)
        path = os.path.join(self.root, *pkg.split('.'), base + '.mako')
        with open(path) as f:
            src = f.read()
        for flt in self.filters:
            src = flt(src)
        return src

    def template(self, name):
        if name not in self._cache:
            code, inherit = compile_template(self.source(name))
            self._cache[name] = (compile(code, f'<template {name}>', 'exec'),
                                 inherit)
        return self._cache[name]

    def render(self, name, **data):
        ctx = Context(data, self)
        self._render_into(name, ctx)
        return ctx.pop_buffer()

    def _render_into(self, name, ctx, nextfn=None):
        code, inherit = self.template(name)

        def body(next_=None):
            env = {'__builtins__': __builtins__}
            env.update(ctx._data)
            exec(code, env)
            env['render'](ctx.write, lambda f: self._render_into(f, ctx),
                          self._call_factory(ctx),
                          lambda m: _ModuleNS(_import(m), ctx),
                          next_)

        if inherit is None:
            body(nextfn and _Next(nextfn))
        else:
            self._render_into(inherit, ctx, lambda: body(nextfn and
                                                          _Next(nextfn)))

    @staticmethod
    def _call_factory(ctx):
        def call(bodyfn, fn, /, **kw):
            ctx._callers.append(_Caller(bodyfn))
            try:
                return fn(**kw)
            finally:
                ctx._callers.pop()
        return call


def _import(name):
    if name not in sys.modules:
        __import__(name)
    return sys.modules[name]
