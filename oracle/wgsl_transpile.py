"""WGSL -> C++ transpiler for the reference's compute passes (test infrastructure only).

The reference's solver kernels are WGSL compute shaders (src/rainbow_fmm.wgsl)
run by wgpu on Vulkan, which this environment cannot host.  This module reads
that shader source and mechanically translates its compute entry points, and
every function they call, into C++ over a small vector runtime
(``wgsl_runtime.hpp``), so the reference's own expressions, loop orders,
constants and control flow run on the host CPU.  The translation is emitted
under ``oracle/_ref/`` at build time; no reference source is stored in this
repository.

Semantics the translation keeps:
  * WGSL abstract-numeric constant expressions (untyped literals and
    operations on them) are folded in binary64 / arbitrary-precision integers
    as the WGSL specification defines, then converted to f32 once;
  * f32 arithmetic stays binary32, left to right as written (the output is
    compiled with -ffp-contract=off);
  * i32 arithmetic wraps (compiled with -fwrapv), f32 -> integer conversions
    saturate, integer <-> integer conversions reinterpret bits;
  * builtins whose precision WGSL leaves to the implementation (inverseSqrt,
    dot, length, normalize, exp, pow, sin, cos, atan2) take one fixed
    definition from ``wgsl_runtime.hpp``.

Supported subset: what the compute half of the shader uses -- structs,
module constants, uniform/storage bindings, functions, let/var/const,
if/else, for, loop, break, continue, return, (compound) assignment,
increment/decrement, vector constructors, single-component and read
swizzles, vector/array indexing, atomics.  Vertex/fragment stages and
texture/sampler bindings are not translated.
"""
from __future__ import annotations

import re
import struct
import sys

# ----------------------------------------------------------------- tokenizer

_TOKEN_RE = re.compile(
    r"""
    (?P<ws>\s+)
  | (?P<lcomment>//[^\n]*)
  | (?P<bcomment>/\*.*?\*/)
  | (?P<num>0[xX][0-9a-fA-F]+[iu]?
           |(?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?[fh]?
           |\d+[eE][+-]?\d+[fh]?
           |\d+[iuf]?)
  | (?P<id>[A-Za-z_][A-Za-z0-9_]*)
  | (?P<op><<=|>>=|->|<=|>=|==|!=|&&|\|\||\+\+|--|\+=|-=|\*=|/=|%=|&=|\|=|\^=|<<|>>
           |[-+*/%<>=!&|^~(){}\[\],;:.@])
    """,
    re.VERBOSE | re.DOTALL,
)


def tokenize(src: str):
    toks, pos = [], 0
    while pos < len(src):
        m = _TOKEN_RE.match(src, pos)
        if m is None:
            raise SyntaxError("wgsl: cannot tokenize at %r" % src[pos:pos + 30])
        pos = m.end()
        kind = m.lastgroup
        if kind in ("ws", "lcomment", "bcomment"):
            continue
        toks.append((kind, m.group(kind)))
    toks.append(("eof", ""))
    return toks


# -------------------------------------------------------------------- parser

_TEMPLATED = {"vec2", "vec3", "vec4", "array", "atomic", "ptr", "mat2x2", "mat3x3", "mat4x4",
              "texture_2d"}
_VEC_ALIAS = {"vec2f": ("vec", 2, "f32"), "vec3f": ("vec", 3, "f32"), "vec4f": ("vec", 4, "f32"),
              "vec2u": ("vec", 2, "u32"), "vec3u": ("vec", 3, "u32"), "vec4u": ("vec", 4, "u32"),
              "vec2i": ("vec", 2, "i32"), "vec3i": ("vec", 3, "i32"), "vec4i": ("vec", 4, "i32")}
_SCALARS = {"f32", "i32", "u32", "bool"}

# Binary operator precedence (higher binds tighter).  WGSL forbids the
# ambiguous mixes C allows, so one table serves.
_BIN_PREC = {
    "||": 1, "&&": 2, "|": 3, "^": 4, "&": 5,
    "==": 6, "!=": 6, "<": 7, ">": 7, "<=": 7, ">=": 7,
    "<<": 8, ">>": 8, "+": 9, "-": 9, "*": 10, "/": 10, "%": 10,
}


class Parser:
    def __init__(self, src: str):
        self.t = tokenize(src)
        self.i = 0
        self.structs = {}     # name -> [(field, type)]
        self.consts = []      # (name, type|None, expr)
        self.globals = []     # (name, address space, type)
        self.funcs = {}       # name -> dict

    # token helpers
    def peek(self, k=0):
        return self.t[self.i + k]

    def next(self):
        tok = self.t[self.i]
        self.i += 1
        return tok

    def accept(self, val):
        if self.t[self.i][1] == val and self.t[self.i][0] in ("op", "id"):
            self.i += 1
            return True
        return False

    def expect(self, val):
        tok = self.next()
        if tok[1] != val:
            raise SyntaxError("wgsl: expected %r, got %r near token %d" % (val, tok[1], self.i))
        return tok

    def ident(self):
        tok = self.next()
        if tok[0] != "id":
            raise SyntaxError("wgsl: expected identifier, got %r" % (tok[1],))
        return tok[1]

    # attributes: @name or @name(args) -- returned as {name: [raw tokens]}
    def attributes(self):
        attrs = {}
        while self.peek()[1] == "@":
            self.next()
            name = self.ident()
            args = []
            if self.peek()[1] == "(":
                self.next()
                depth = 1
                while depth:
                    tok = self.next()
                    if tok[1] == "(":
                        depth += 1
                    elif tok[1] == ")":
                        depth -= 1
                        if depth == 0:
                            break
                    args.append(tok[1])
            attrs[name] = args
        return attrs

    # types
    def close_angle(self):
        tok = self.peek()
        if tok[1] == ">":
            self.next()
        elif tok[1] == ">>":
            self.t[self.i] = ("op", ">")
        elif tok[1] == ">=":
            self.t[self.i] = ("op", "=")
        else:
            raise SyntaxError("wgsl: expected '>' in a type, got %r" % (tok[1],))

    def type_(self):
        name = self.ident()
        if name in _VEC_ALIAS:
            return _VEC_ALIAS[name]
        if name in _SCALARS:
            return ("scalar", name)
        if name in _TEMPLATED and self.peek()[1] == "<":
            self.next()
            if name.startswith("vec"):
                elem = self.type_()
                self.close_angle()
                return ("vec", int(name[3]), elem[1])
            if name == "atomic":
                elem = self.type_()
                self.close_angle()
                return ("atomic", elem[1])
            if name == "array":
                elem = self.type_()
                size = None
                if self.accept(","):
                    size = self.expr(8)  # no relational operators inside <...>
                self.close_angle()
                return ("array", elem, size)
            depth = 1  # other templated types: skipped (textures, pointers)
            while depth:
                tok = self.next()
                if tok[1] == "<":
                    depth += 1
                elif tok[1] == ">":
                    depth -= 1
                elif tok[1] == ">>":
                    depth -= 2
            return ("opaque", name)
        if name in self.structs:
            return ("struct", name)
        return ("opaque", name)

    # module
    def module(self):
        while self.peek()[0] != "eof":
            attrs = self.attributes()
            tok = self.peek()
            if tok[1] == "struct":
                self.next()
                name = self.ident()
                self.expect("{")
                fields = []
                while not self.accept("}"):
                    self.attributes()
                    fname = self.ident()
                    self.expect(":")
                    fields.append((fname, self.type_()))
                    self.accept(",")
                self.structs[name] = fields
                self.accept(";")
            elif tok[1] == "const":
                self.next()
                name = self.ident()
                ty = None
                if self.accept(":"):
                    ty = self.type_()
                self.expect("=")
                self.consts.append((name, ty, self.expr()))
                self.expect(";")
            elif tok[1] == "var":
                self.next()
                space = []
                if self.peek()[1] == "<":
                    self.next()
                    while not self.accept(">"):
                        tok2 = self.next()
                        if tok2[1] != ",":
                            space.append(tok2[1])
                name = self.ident()
                self.expect(":")
                ty = self.type_()
                self.expect(";")
                self.globals.append((name, tuple(space), ty, attrs))
            elif tok[1] == "fn":
                self.next()
                name = self.ident()
                self.expect("(")
                params = []
                while not self.accept(")"):
                    pattrs = self.attributes()
                    pname = self.ident()
                    self.expect(":")
                    params.append((pname, self.type_(), pattrs))
                    self.accept(",")
                ret = None
                if self.accept("->"):
                    self.attributes()
                    ret = self.type_()
                body = self.block()
                self.funcs[name] = {"name": name, "params": params, "ret": ret, "body": body,
                                    "attrs": attrs}
            else:
                raise SyntaxError("wgsl: unexpected module-scope token %r" % (tok[1],))

    # statements
    def block(self):
        self.expect("{")
        stmts = []
        while not self.accept("}"):
            stmts.append(self.statement())
        return ("block", stmts)

    def statement(self):
        tok = self.peek()
        v = tok[1]
        if tok[0] == "op" and v == "{":
            return self.block()
        if tok[0] == "id":
            if v in ("let", "var", "const"):
                s = self.decl()
                self.expect(";")
                return s
            if v == "return":
                self.next()
                e = None if self.peek()[1] == ";" else self.expr()
                self.expect(";")
                return ("return", e)
            if v == "if":
                return self.if_()
            if v == "for":
                self.next()
                self.expect("(")
                init = None if self.peek()[1] == ";" else self.simple_statement()
                self.expect(";")
                cond = None if self.peek()[1] == ";" else self.expr()
                self.expect(";")
                upd = None if self.peek()[1] == ")" else self.simple_statement()
                self.expect(")")
                return ("for", init, cond, upd, self.block())
            if v == "loop":
                self.next()
                return ("loop", self.block())
            if v == "while":
                self.next()
                cond = self.expr()
                return ("for", None, cond, None, self.block())
            if v in ("break", "continue"):
                self.next()
                self.expect(";")
                return (v,)
        s = self.simple_statement()
        self.expect(";")
        return s

    def decl(self):
        kind = self.next()[1]
        name = self.ident()
        ty = None
        if self.accept(":"):
            ty = self.type_()
        init = None
        if self.accept("="):
            init = self.expr()
        return ("decl", kind, name, ty, init)

    def simple_statement(self):
        if self.peek()[1] in ("let", "var", "const"):
            return self.decl()
        lhs = self.expr()
        op = self.peek()[1]
        if op in ("=", "+=", "-=", "*=", "/=", "%=", "&=", "|=", "^=", "<<=", ">>="):
            self.next()
            return ("assign", op, lhs, self.expr())
        if op in ("++", "--"):
            self.next()
            return ("incr", op, lhs)
        return ("expr", lhs)

    def if_(self):
        self.expect("if")
        cond = self.expr()
        then = self.block()
        other = None
        if self.accept("else"):
            other = self.if_() if self.peek()[1] == "if" else self.block()
        return ("if", cond, then, other)

    # expressions
    def expr(self, min_prec=1):
        lhs = self.unary()
        while True:
            op = self.peek()[1]
            if self.peek()[0] != "op" or op not in _BIN_PREC or _BIN_PREC[op] < min_prec:
                return lhs
            self.next()
            rhs = self.expr(_BIN_PREC[op] + 1)
            lhs = ("bin", op, lhs, rhs)

    def unary(self):
        tok = self.peek()
        if tok[0] == "op" and tok[1] in ("-", "!", "~", "&", "*"):
            self.next()
            return ("un", tok[1], self.unary())
        return self.postfix(self.primary())

    def postfix(self, e):
        while True:
            v = self.peek()[1]
            if v == "[":
                self.next()
                idx = self.expr()
                self.expect("]")
                e = ("idx", e, idx)
            elif v == "." and self.peek()[0] == "op":
                self.next()
                e = ("mem", e, self.ident())
            else:
                return e

    def args(self):
        self.expect("(")
        out = []
        while not self.accept(")"):
            out.append(self.expr())
            self.accept(",")
        return out

    def primary(self):
        kind, v = self.next()
        if kind == "num":
            return parse_number(v)
        if kind == "op" and v == "(":
            e = self.expr()
            self.expect(")")
            return ("paren", e)
        if kind == "id":
            if v in ("true", "false"):
                return ("lit", "bool", v == "true", v)
            if v in _TEMPLATED and self.peek()[1] == "<":
                self.i -= 1
                ty = self.type_()
                return ("ctor", ty, self.args())
            if v in _VEC_ALIAS or v in _SCALARS:
                ty = _VEC_ALIAS.get(v, ("scalar", v))
                return ("ctor", ty, self.args())
            if v in ("vec2", "vec3", "vec4") and self.peek()[1] == "(":
                return ("ctor", ("vec", int(v[3]), None), self.args())
            if self.peek()[1] == "(":
                if v in self.structs:
                    return ("ctor", ("struct", v), self.args())
                return ("call", v, self.args())
            return ("id", v)
        raise SyntaxError("wgsl: unexpected token %r in an expression" % (v,))


def parse_number(text: str):
    t = text
    if t[:2] in ("0x", "0X"):
        suffix = t[-1] if t[-1] in "iu" else ""
        val = int(t[:-1] if suffix else t, 16)
        return ("lit", {"": "aint", "i": "i32", "u": "u32"}[suffix], val, text)
    if t[-1] in "fh":
        return ("lit", "f32", float(t[:-1]), text)
    if t[-1] in "iu" and re.fullmatch(r"\d+[iu]", t):
        return ("lit", {"i": "i32", "u": "u32"}[t[-1]], int(t[:-1]), text)
    if re.fullmatch(r"\d+", t):
        return ("lit", "aint", int(t), text)
    return ("lit", "afloat", float(t), text)


# ------------------------------------------------------------------- emitter

_SCALAR_CPP = {"f32": "float", "i32": "int32_t", "u32": "uint32_t", "bool": "bool"}
_SWIZZLE = re.compile(r"[xyzw]{1,4}")
_BUILTINS = {
    "abs", "min", "max", "clamp", "floor", "ceil", "round", "fract", "sqrt", "inverseSqrt",
    "length", "normalize", "dot", "cross", "mix", "smoothstep", "select", "exp", "exp2", "log",
    "log2", "pow", "sin", "cos", "tan", "atan", "atan2", "any", "all", "sign", "step", "trunc",
    "atomicAdd", "atomicSub", "atomicLoad", "atomicStore", "atomicMax", "atomicMin",
    "arrayLength", "distance",
}


def f32_of(x: float) -> float:
    """Round a binary64 value to binary32 (round to nearest even)."""
    return struct.unpack("<f", struct.pack("<f", x))[0]


def int_literal(v: int) -> str:
    """An abstract integer as C++: int in i32 range (C++ then converts it like
    WGSL concretises it), u32 above, refused beyond (C++ would widen to 64
    bits where WGSL cannot)."""
    if -(1 << 31) <= v < (1 << 31):
        return "(%d)" % v
    if 0 <= v < (1 << 32):
        return "(%du)" % v
    raise ValueError("wgsl: integer constant %d outside i32/u32" % v)


def f32_literal(x: float) -> str:
    v = f32_of(x)
    if v != v or v in (float("inf"), float("-inf")):
        raise ValueError("wgsl: non-finite constant")
    return "(%sf)" % float.hex(v)


class Emitter:
    def __init__(self, p: Parser):
        self.p = p
        self.abstract_consts = {}  # untyped module constants with an abstract value
        for name, ty, e in p.consts:
            if ty is None:
                v = self.fold(e)
                if v is not None:
                    self.abstract_consts[name] = v

    # types
    def ctype(self, ty):
        k = ty[0]
        if k == "scalar":
            return _SCALAR_CPP[ty[1]]
        if k == "vec":
            return "wgsl::vec<%s, %d>" % (_SCALAR_CPP[ty[2]], ty[1])
        if k == "struct":
            return "T_" + ty[1]
        if k == "atomic":
            return _SCALAR_CPP[ty[1]]
        if k == "array":
            if ty[2] is None:
                return self.ctype(ty[1]) + "*"
            return "wgsl::arr<%s, %s>" % (self.ctype(ty[1]), self.expr(ty[2]))
        raise TypeError("wgsl: type %r is not translated" % (ty,))

    # abstract constant folding: returns ("aint"|"afloat", value) or None
    def fold(self, e):
        k = e[0]
        if k == "lit" and e[1] in ("aint", "afloat"):
            return (e[1], e[2])
        if k == "paren":
            return self.fold(e[1])
        if k == "id" and e[1] in getattr(self, "abstract_consts", {}):
            return self.abstract_consts[e[1]]
        if k == "un" and e[1] == "-":
            v = self.fold(e[2])
            return None if v is None else (v[0], -v[1])
        if k == "bin" and e[1] in ("+", "-", "*", "/"):
            a, b = self.fold(e[2]), self.fold(e[3])
            if a is None or b is None:
                return None
            if a[0] == "aint" and b[0] == "aint":
                x, y = a[1], b[1]
                if e[1] == "/":
                    if y == 0:
                        return None
                    q = abs(x) // abs(y)
                    return ("aint", q if (x >= 0) == (y >= 0) else -q)
                return ("aint", {"+": x + y, "-": x - y, "*": x * y}[e[1]])
            x, y = float(a[1]), float(b[1])
            return ("afloat", {"+": x + y, "-": x - y, "*": x * y, "/": x / y}[e[1]])
        return None

    def expr(self, e):
        v = self.fold(e)
        if v is not None:
            if v[0] == "afloat":
                return f32_literal(v[1])
            return int_literal(v[1])
        k = e[0]
        if k == "lit":
            kind, val = e[1], e[2]
            if kind == "bool":
                return "true" if val else "false"
            if kind == "f32":
                return f32_literal(val)
            if kind == "u32":
                return "%du" % val
            return "int32_t(%d)" % val
        if k == "paren":
            return self.expr(e[1])
        if k == "id":
            return "w_" + e[1]
        if k == "un":
            if e[1] == "&":
                return "(&%s)" % self.expr(e[2])
            if e[1] == "*":
                return "(*%s)" % self.expr(e[2])
            return "(%s%s)" % (e[1], self.expr(e[2]))
        if k == "bin":
            a, b = self.expr(e[2]), self.expr(e[3])
            if e[1] == "%":
                return "wgsl::mod(%s, %s)" % (a, b)
            return "(%s %s %s)" % (a, e[1], b)
        if k == "idx":
            return "%s[%s]" % (self.expr(e[1]), self.expr(e[2]))
        if k == "mem":
            name = e[2]
            base = self.expr(e[1])
            if _SWIZZLE.fullmatch(name):
                idx = ["xyzw".index(ch) for ch in name]
                if len(idx) == 1:
                    return "%s.v[%d]" % (base, idx[0])
                return "wgsl::swizzle<%s>(%s)" % (", ".join(map(str, idx)), base)
            return "%s.%s" % (base, name)
        if k == "ctor":
            ty = e[1]
            args = [self.expr(a) for a in e[2]]
            if ty[0] == "struct":
                return "T_%s{%s}" % (ty[1], ", ".join(args))
            if ty[0] == "scalar":
                if len(args) != 1:
                    raise TypeError("wgsl: scalar constructor with %d arguments" % len(args))
                return "wgsl::convert<%s>(%s)" % (_SCALAR_CPP[ty[1]], args[0])
            if ty[0] == "vec":
                if ty[2] is None:
                    raise TypeError("wgsl: vector constructor without an element type")
                return "wgsl::make<%s, %d>(%s)" % (_SCALAR_CPP[ty[2]], ty[1], ", ".join(args))
            raise TypeError("wgsl: constructor of %r is not translated" % (ty,))
        if k == "call":
            name = e[1]
            args = ", ".join(self.expr(a) for a in e[2])
            if name in _BUILTINS:
                return "wgsl::%s(%s)" % (name, args)
            return "w_%s(%s)" % (name, args)
        raise TypeError("wgsl: expression %r is not translated" % (k,))

    def stmt(self, s, ind):
        pad = "  " * ind
        k = s[0]
        if k == "block":
            return pad + "{\n" + "".join(self.stmt(x, ind + 1) for x in s[1]) + pad + "}\n"
        if k in ("decl", "assign", "incr", "expr"):
            return pad + self.simple(s) + ";\n"
        if k == "return":
            return pad + ("return %s;\n" % self.expr(s[1]) if s[1] is not None else "return;\n")
        if k == "if":
            out = pad + "if (%s) " % self.expr(s[1]) + self.stmt(s[2], ind).lstrip()
            if s[3] is not None:
                out = out.rstrip("\n") + " else " + self.stmt(s[3], ind).lstrip()
            return out
        if k == "for":
            init = self.simple(s[1]) if s[1] is not None else ""
            cond = self.expr(s[2]) if s[2] is not None else ""
            upd = self.simple(s[3]) if s[3] is not None else ""
            return pad + "for (%s; %s; %s) " % (init, cond, upd) + self.stmt(s[4], ind).lstrip()
        if k == "loop":
            return pad + "for (;;) " + self.stmt(s[1], ind).lstrip()
        if k in ("break", "continue"):
            return pad + k + ";\n"
        raise TypeError("wgsl: statement %r is not translated" % (k,))

    def simple(self, s):
        k = s[0]
        if k == "decl":
            _, kind, name, ty, init = s
            if kind == "const" and ty is None:
                # A function-scope abstract constant would need scoped folding;
                # the translated shader has none, so refuse rather than guess.
                raise NotImplementedError("wgsl: function-scope untyped const %r" % name)
            if ty is not None:
                ct = self.ctype(ty)
                if init is None:
                    return "%s w_%s{}" % (ct, name)
                return "%s w_%s = wgsl::convert<%s>(%s)" % (ct, name, ct, self.expr(init))
            return "auto w_%s = %s" % (name, self.expr(init))
        if k == "assign":
            return "%s %s %s" % (self.expr(s[2]), s[1], self.expr(s[3]))
        if k == "incr":
            return "%s%s" % (self.expr(s[2]), s[1])
        if k == "expr":
            return self.expr(s[1])
        raise TypeError("wgsl: simple statement %r" % (k,))

    # call graph from the compute entry points
    def reachable(self):
        seen, order = set(), []

        def calls(node, acc):
            if isinstance(node, tuple):
                if node and node[0] == "call" and node[1] in self.p.funcs:
                    acc.add(node[1])
                for x in node:
                    calls(x, acc)
            elif isinstance(node, list):
                for x in node:
                    calls(x, acc)

        def visit(name):
            if name in seen:
                return
            seen.add(name)
            acc = set()
            calls(self.p.funcs[name]["body"], acc)
            for c in sorted(acc):
                visit(c)
            order.append(name)

        for name, f in self.p.funcs.items():
            if "compute" in f["attrs"]:
                visit(name)
        return order

    def module(self):
        p = self.p
        out = ["// Generated by oracle/wgsl_transpile.py from the reference shader; do not edit.\n",
               "// Compute entry points and their callees only.\n",
               "#include <cstdint>\n#include \"wgsl_runtime.hpp\"\n\n"]
        for name, fields in p.structs.items():
            try:
                body = "".join("  %s %s;\n" % (self.ctype(t), f) for f, t in fields)
            except TypeError:
                continue  # stage-interface structs (vertex outputs) are not translated
            out.append("struct T_%s {\n%s};\n" % (name, body))
        out.append("\n")
        for name, ty, e in p.consts:
            if ty is None:
                continue  # folded at each use
            ct = self.ctype(ty)
            out.append("static const %s w_%s = wgsl::convert<%s>(%s);\n" % (ct, name, ct, self.expr(e)))
        out.append("\n")
        for name, space, ty, attrs in p.globals:
            if ty[0] == "opaque":
                continue  # textures and samplers
            out.append("static %s w_%s{};  // var<%s>\n" % (self.ctype(ty), name, ", ".join(space)))
        out.append("\n")
        order = self.reachable()
        sigs = {}
        for name in order:
            f = p.funcs[name]
            ret = "void" if f["ret"] is None else self.ctype(f["ret"])
            params = ", ".join("%s w_%s" % (self.ctype(t), n) for n, t, _ in f["params"])
            sigs[name] = "static %s w_%s(%s)" % (ret, name, params)
            out.append(sigs[name] + ";\n")
        out.append("\n")
        for name in order:
            out.append(sigs[name] + " " + self.stmt(p.funcs[name]["body"], 0).lstrip() + "\n")
        # entry-point table: name, workgroup size
        out.append("struct wgsl_entry { const char *name; void (*fn)(wgsl::vec<uint32_t, 3>); uint32_t wg; };\n")
        out.append("static const wgsl_entry wgsl_entries[] = {\n")
        for name in order:
            f = p.funcs[name]
            if "compute" in f["attrs"]:
                wg = int("".join(f["attrs"].get("workgroup_size", ["1"])).split(",")[0])
                out.append('  {"%s", w_%s, %du},\n' % (name, name, wg))
        out.append("};\n")
        return "".join(out)


def transpile(src: str) -> str:
    p = Parser(src)
    p.module()
    return Emitter(p).module()


def entry_points(src: str):
    p = Parser(src)
    p.module()
    return [n for n, f in p.funcs.items() if "compute" in f["attrs"]]


if __name__ == "__main__":
    with open(sys.argv[1]) as fh:
        sys.stdout.write(transpile(fh.read()))
