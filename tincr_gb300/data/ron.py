"""Minimal reader for the subset of RON (Rusty Object Notation) used by tincr's parameter files.

tincr stores its Slater-Koster tables, pseudo-atom data and repulsive potentials as RON
(`src/param/slaterkoster/**/*.ron`, `src/param/repulsive_potential/reppot_tables/*.ron`, read by
`src/initialization/parameters.rs:91-113`, `:191-213`, `:301-321` through `ron::de::from_str`).
The files use: anonymous structs `( key: value, ... )`, maps `{ k: v, ... }`, lists `[ ... ]`,
tuples `( a, b, c )`, numbers, `inf`, and double-quoted strings.  Structs become dicts,
tuples become Python tuples, maps become dicts keyed by the parsed key.
"""

import re

_TOKEN = re.compile(
    r"""\s*(?:
        (?P<num>[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?)
      | (?P<str>"(?:[^"\\]|\\.)*")
      | (?P<ident>[A-Za-z_][A-Za-z_0-9]*)
      | (?P<punct>[()\[\]{}:,])
    )""",
    re.X,
)


def _tokenize(text):
    pos = 0
    out = []
    n = len(text)
    while pos < n:
        m = _TOKEN.match(text, pos)
        if not m:
            rest = text[pos:].strip()
            if not rest:
                break
            raise ValueError("RON: cannot tokenize near %r" % text[pos:pos + 40])
        pos = m.end()
        kind = m.lastgroup
        out.append((kind, m.group(kind)))
    return out


class _Parser:
    def __init__(self, tokens):
        self.t = tokens
        self.i = 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, val=None):
        tok = self.t[self.i]
        if val is not None and tok[1] != val:
            raise ValueError("RON: expected %r got %r" % (val, tok[1]))
        self.i += 1
        return tok

    def value(self):
        kind, val = self.peek()
        if kind == "num":
            self.take()
            if re.fullmatch(r"[-+]?\d+", val):
                return int(val)
            return float(val)
        if kind == "str":
            self.take()
            return val[1:-1]
        if kind == "ident":
            self.take()
            if val == "inf":
                return float("inf")
            if val in ("NaN", "nan"):
                return float("nan")
            if val == "true":
                return True
            if val == "false":
                return False
            if val == "None":
                return None
            if val == "Some":
                self.take("(")
                v = self.value()
                self.take(")")
                return v
            # a named struct like Foo( ... )
            if self.peek()[1] == "(":
                return self.value()
            return val
        if val == "[":
            self.take("[")
            items = []
            while self.peek()[1] != "]":
                items.append(self.value())
                if self.peek()[1] == ",":
                    self.take(",")
            self.take("]")
            return items
        if val == "{":
            self.take("{")
            d = {}
            while self.peek()[1] != "}":
                k = self.value()
                self.take(":")
                d[k] = self.value()
                if self.peek()[1] == ",":
                    self.take(",")
            self.take("}")
            return d
        if val == "(":
            self.take("(")
            # struct if "ident :" follows
            if self.peek()[0] == "ident" and self.peek(1)[1] == ":":
                d = {}
                while self.peek()[1] != ")":
                    _, key = self.take()
                    self.take(":")
                    d[key] = self.value()
                    if self.peek()[1] == ",":
                        self.take(",")
                self.take(")")
                return d
            items = []
            while self.peek()[1] != ")":
                items.append(self.value())
                if self.peek()[1] == ",":
                    self.take(",")
            self.take(")")
            return tuple(items)
        raise ValueError("RON: unexpected token %r" % (val,))


def loads(text):
    """Parse RON text into Python objects."""
    p = _Parser(_tokenize(text))
    v = p.value()
    return v
