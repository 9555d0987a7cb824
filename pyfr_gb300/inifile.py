"""Minimal INI configuration with the accessors the solver code uses
(``get``, ``getint``, ``getfloat``, ``getbool``, ``getexpr``, ``items``,
``items_as``, ``hasopt``, ``set``), following the interface of
``pyfr/inifile.py:31-161``.  Expressions may reference ``[constants]``;
``getexpr`` substitutes them textually, as the reference does.
"""

from configparser import ConfigParser
import io
import re


class Inifile:
    def __init__(self, inistr=None):
        self._cp = ConfigParser(inline_comment_prefixes=[';'],
                                interpolation=None)
        self._cp.optionxform = str
        if inistr:
            self._cp.read_string(inistr)

    @classmethod
    def load(cls, path):
        with open(path) as f:
            return cls(f.read())

    def set(self, section, option, value):
        if not self._cp.has_section(section):
            self._cp.add_section(section)
        self._cp.set(section, option, str(value))

    def hassect(self, section):
        return self._cp.has_section(section)

    def hasopt(self, section, option):
        return self._cp.has_option(section, option)

    _NODEF = object()

    def get(self, section, option, default=_NODEF):
        if self._cp.has_option(section, option):
            return self._cp.get(section, option)
        if default is self._NODEF:
            raise KeyError(f'Missing option {option!r} in [{section}]')
        return None if default is None else str(default)

    def getint(self, section, option, default=_NODEF):
        v = self.get(section, option, default)
        return None if v is None else int(v)

    def getfloat(self, section, option, default=_NODEF):
        v = self.get(section, option, default)
        return None if v is None else float(v)

    def getbool(self, section, option, default=_NODEF):
        v = self.get(section, option, default)
        if v is None:
            return None
        return v.strip().lower() in ('1', 'true', 'yes', 'on')

    def items(self, section):
        if not self._cp.has_section(section):
            return {}
        return dict(self._cp.items(section))

    def items_as(self, section, type):
        out = {}
        for k, v in self.items(section).items():
            try:
                out[k] = type(v)
            except ValueError:
                pass
        return out

    def getexpr(self, section, option, default=_NODEF, subs={}):
        expr = self.get(section, option, default)
        if expr is None:
            return None

        subs = self.items('constants') | dict(subs)
        if subs:
            pat = r'\b(' + '|'.join(map(re.escape, sorted(subs, key=len,
                                                         reverse=True))) + r')\b'
            expr = re.sub(pat, lambda m: f'({subs[m[1]]})', expr)
        return expr

    def tostr(self):
        buf = io.StringIO()
        self._cp.write(buf)
        return buf.getvalue()
