"""Reader for the Lua data files that gdtk's pre-processors write.

TEST INFRASTRUCTURE: used by the oracle (oracle/__init__.py) only.  The product library
has its own reader in C++ (gdtk_gb300/csrc/lua_table.cpp); keeping two independent
readers means a parsing mistake shows up as an oracle/product mismatch.

The files are Lua chunks made of assignment statements whose right-hand sides are
literals and table constructors, e.g. (prep_gas.lua / prep_chem.lua output)

    species = {[0]='N2', [1]='O2', }
    db['N2'].thermoCoeffs = { nsegments = 3, T_break_points = {200.0, 1000.0}, ... }
    reaction[1] = { frc = {model='Arrhenius', A=7.0e15, n=-1.6, C=113200.0}, ... }

Tables are returned as dicts; integer keys stay ints (the implicit array part of a
constructor is numbered from 1, as in Lua).
"""
import re

_TOKEN = re.compile(r"""
    (?P<ws>\s+|--\[(?P<eq>=*)\[.*?\](?P=eq)\]|--[^\n]*)
  | (?P<num>0[xX][0-9a-fA-F]+|(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)
  | (?P<str>'(?:\\.|[^'\\])*'|"(?:\\.|[^"\\])*")
  | (?P<name>[A-Za-z_][A-Za-z_0-9]*)
  | (?P<op>\.\.|==|[=,;{}\[\]().\-+*/])
""", re.S | re.X)


def _tokens(text):
    pos = 0
    out = []
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            raise ValueError("cannot tokenise Lua input at offset %d: %r" % (pos, text[pos:pos + 20]))
        pos = m.end()
        if m.group('ws') is not None:
            continue
        for kind in ('num', 'str', 'name', 'op'):
            v = m.group(kind)
            if v is not None:
                out.append((kind, v))
                break
    out.append(('eof', None))
    return out


class _Parser:
    def __init__(self, text):
        self.t = _tokens(text)
        self.i = 0
        self.env = {}

    def peek(self):
        return self.t[self.i]

    def take(self, val=None):
        tok = self.t[self.i]
        if val is not None and tok[1] != val:
            raise ValueError("expected %r, found %r" % (val, tok[1]))
        self.i += 1
        return tok

    def chunk(self):
        while self.peek()[0] != 'eof':
            if self.peek()[1] == ';':
                self.take()
                continue
            self.statement()
        return self.env

    def statement(self):
        kind, name = self.take()
        if kind != 'name':
            raise ValueError("statement must start with a name, found %r" % name)
        keys = []
        while self.peek()[1] in ('.', '['):
            if self.take()[1] == '.':
                keys.append(self.take()[1])
            else:
                keys.append(self.expr())
                self.take(']')
        self.take('=')
        value = self.expr()
        if not keys:
            self.env[name] = value
            return
        target = self.env[name]
        for k in keys[:-1]:
            target = target[k]
        target[keys[-1]] = value

    def expr(self):
        kind, v = self.peek()
        if v == '-':
            self.take()
            return -self.expr()
        if v == '{':
            return self.table()
        self.take()
        if kind == 'num':
            if v.lower().startswith('0x'):
                return int(v, 16)
            if re.fullmatch(r'\d+', v):
                return int(v)
            return float(v)
        if kind == 'str':
            return bytes(v[1:-1], 'utf-8').decode('unicode_escape')
        if kind == 'name':
            if v == 'true':
                return True
            if v == 'false':
                return False
            if v == 'nil':
                return None
            return self.env[v]
        raise ValueError("unexpected token %r" % v)

    def table(self):
        self.take('{')
        out = {}
        n = 1
        while self.peek()[1] != '}':
            kind, v = self.peek()
            if v == '[':
                self.take()
                key = self.expr()
                self.take(']')
                self.take('=')
                out[key] = self.expr()
            elif kind == 'name' and self.t[self.i + 1][1] == '=':
                self.take()
                self.take('=')
                out[v] = self.expr()
            else:
                out[n] = self.expr()
                n += 1
            if self.peek()[1] in (',', ';'):
                self.take()
        self.take('}')
        return out


def read_lua_file(path):
    with open(path) as f:
        return _Parser(f.read()).chunk()


def array(tab):
    """Values of a Lua sequence {1: a, 2: b, ...} (or one written from [0]) in index order."""
    keys = sorted(k for k in tab if isinstance(k, int))
    return [tab[k] for k in keys]
