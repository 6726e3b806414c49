"""Build recipe for oracle/_ref/librust_ref.so: cantucci's own Rust source for
the estimator and the mesher, translated mechanically into C++ and compiled
(test infrastructure, like the rest of oracle/).

The reference is Rust (nightly, x86-64 SSE4.1 only) and this image has no
Rust toolchain, so its code cannot be built as Rust.  The part on the hot
path is plain arithmetic, though, and this recipe turns its source text into
C++ without a human restating it:

  src/shape/mandelbulb.rs   Mandelbulb, new, min_distance_from, rotate,
                            rotate_on_z_axis, rotate_inner_px_generic,
                            rotate_inner_p8_scalar, Vec3 and its operators
  src/shape/sphere.rs       Sphere, new, min_distance_from, contains
  src/shape/mod.rs          Shape::contains (the trait's default)
  src/mesh/buffer.rs        MeshBuffer, generate_for_box, naive_surface_nets,
                            Timings
  src/mesh/mod.rs           Vertex
  src/math.rs               lerp and Lerp for Point3<f32>
  src/util/grid.rs          GridTable, fill_with, Index
  src/util/iter.rs          cube, CubeIter, Iterator::next
  src/octree/mod.rs         Span

It reads those files where they lie in the reference tree (the directory
named by the CANTUCCI_REFERENCE environment variable), picks the items above
out of them, and translates a small subset of Rust: `let` (with shadowing),
blocks and `if`/`match` as values (GCC statement expressions), closures
(lambdas), `for` over ranges and iterators, struct and tuple literals,
method calls (`a.m(b)` -> `m_m(a, b)`), associated functions
(`T::f` -> `T__f`), operator traits (-> C++ operators), `as` casts, `assert!`
(-> a thrown rsref::Panic) and `#[cfg]` evaluated for x86-64 with SSE4.1
(the reference builds with -C target-cpu=native).  Every unsuffixed float
literal is f32: the translated items contain no f64, which the recipe checks.
Arithmetic is emitted exactly as written, fully parenthesised in Rust's own
precedence, and compiled with -ffp-contract=off and no FMA, so every f32 sum
and product rounds on its own, as rustc compiles it.  Anything outside the
subset stops the build with an error instead of being guessed.

What the reference takes from outside its tree comes from rust_shim.h: Rust
std's f32 methods (glibc libm, sqrtss, LLVM's powi expansion) and cgmath
0.18.0's Point3/Vector3 arithmetic (not vendored in the reference).

The translated text and the library are written only under oracle/_ref/
(git-ignored).  The C entry points are

    int rustref_de(const rustref_shape*, const float* xyz, uint64 n, float* out)
    int rustref_contains(const rustref_shape*, const float* xyz, uint64 n, uint8* out)
    int rustref_generate_for_box(const rustref_shape*, const float span[6], uint32 res,
                                 float* vertices7, uint64 vcap, uint32* indices, uint64 icap,
                                 uint64* nv, uint64* ni, float* dists, uint32* points)

returning 0, or 1 when generate_for_box's or Mandelbulb::new's assert! fails,
3 when lerp's assert! fails (the reference panics there), 4 on an
out-of-range index, 2 when an output is too small.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "librust_ref.so")
SHIM = os.path.join(HERE, "rust_shim.h")

# Integer powers instantiated from the const-generic Mandelbulb<const P: u8>.
POWERS = (2, 3, 4, 5, 6, 7, 8, 9, 10, 12)

# (file, selector).  Selectors: ("struct", name), ("fn", name), ("type", name),
# ("impl", key, [methods] or None for all), ("trait_default", trait, method).
# Order matters only for the structs (emitted in this order).
ITEMS = [
    ("src/octree/mod.rs", ("type", "Span")),
    ("src/mesh/mod.rs", ("struct", "Vertex")),
    ("src/mesh/buffer.rs", ("struct", "MeshBuffer")),
    ("src/mesh/buffer.rs", ("struct", "Timings")),
    ("src/util/grid.rs", ("struct", "GridTable")),
    ("src/util/iter.rs", ("struct", "CubeIter")),
    ("src/shape/mandelbulb.rs", ("struct", "Mandelbulb")),
    ("src/shape/mandelbulb.rs", ("struct", "Vec3")),
    ("src/shape/sphere.rs", ("struct", "Sphere")),
    ("src/util/iter.rs", ("fn", "cube")),
    ("src/util/iter.rs", ("impl", "Iterator for CubeIter", ["next"])),
    ("src/util/grid.rs", ("impl", "GridTable", ["fill_with"])),
    ("src/util/grid.rs", ("impl", "Index for GridTable", ["index"])),
    ("src/math.rs", ("fn", "lerp")),
    ("src/math.rs", ("impl", "Lerp for Point3", ["lerp"])),
    ("src/shape/mod.rs", ("trait_default", "Shape", "contains")),
    ("src/shape/mandelbulb.rs", ("impl", "Mandelbulb", ["new"])),
    ("src/shape/mandelbulb.rs", ("impl", "Shape for Mandelbulb", ["min_distance_from"])),
    ("src/shape/mandelbulb.rs", ("fn", "rotate")),
    ("src/shape/mandelbulb.rs", ("fn", "rotate_on_z_axis")),
    ("src/shape/mandelbulb.rs", ("fn", "rotate_inner_px_generic")),
    ("src/shape/mandelbulb.rs", ("fn", "rotate_inner_p8_scalar")),
    ("src/shape/mandelbulb.rs", ("impl", "Vec3", ["new", "x", "y", "z", "magnitude",
                                                  "is_on_z_axis"])),
    ("src/shape/mandelbulb.rs", ("impl", "Add for Vec3", None)),
    ("src/shape/mandelbulb.rs", ("impl", "Sub for Vec3", None)),
    ("src/shape/mandelbulb.rs", ("impl", "Mul for Vec3", None)),
    ("src/shape/mandelbulb.rs", ("impl", "Mul for f32", None)),
    ("src/shape/sphere.rs", ("impl", "Sphere", ["new"])),
    ("src/shape/sphere.rs", ("impl", "Shape for Sphere", ["min_distance_from", "contains"])),
    ("src/mesh/buffer.rs", ("impl", "MeshBuffer", ["generate_for_box", "naive_surface_nets"])),
]
# Values passed through rsref::rs_observe before they are returned.
OBSERVE_RETURNS = {("GridTable", "fill_with")}

CFG = {"target_arch": {"x86_64"}, "target_feature": {"sse", "sse2", "sse3", "ssse3", "sse4.1",
                                                      "sse4.2"}, "test": False}

CXXFLAGS = ["-O2", "-std=gnu++20", "-fPIC", "-shared", "-msse4.1", "-mno-fma",
            "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-variable",
            "-Wno-unused-but-set-variable", "-Wno-unused-function"]


class TranslateError(Exception):
    pass


def reference_root():
    return os.environ.get("CANTUCCI_REFERENCE")


def available() -> bool:
    root = reference_root()
    return bool(root) and all(os.path.exists(os.path.join(root, f)) for f, _ in ITEMS)


# ---------------------------------------------------------------- lexer
_TOKEN = re.compile(r"""
 (?P<ws>\s+)
|(?P<lcom>//[^\n]*)
|(?P<bcom>/\*.*?\*/)
|(?P<str>"(?:[^"\\]|\\.)*")
|(?P<num>0x[0-9A-Fa-f_]+|0b[01_]+|[0-9][0-9_]*(?:\.[0-9][0-9_]*)?(?:[eE][+-]?[0-9_]+)?
          (?:f32|f64|u8|u16|u32|u64|usize|i8|i16|i32|i64|isize)?)
|(?P<id>[A-Za-z_][A-Za-z0-9_]*)
|(?P<p>::|->|=>|\.\.=|\.\.|==|!=|<=|>=|&&|\|\||\+=|-=|\*=|/=|%=|[-+*/%=<>!&|^.,;:\#()\[\]{}?@$~'])
""", re.X | re.S)


class Tok:
    __slots__ = ("k", "t", "line")

    def __init__(self, k, t, line):
        self.k, self.t, self.line = k, t, line

    def __repr__(self):
        return "%s@%d" % (self.t, self.line)


def lex(text, path):
    toks, pos, line = [], 0, 1
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            raise TranslateError("%s:%d: cannot lex %r" % (path, line, text[pos:pos + 20]))
        k = m.lastgroup
        s = m.group(k)
        if k not in ("ws", "lcom", "bcom"):
            toks.append(Tok(k, s, line))
        line += s.count("\n")
        pos = m.end()
    toks.append(Tok("eof", "", line))
    return toks


# ---------------------------------------------------------------- item skimmer
_CLOSE = {"(": ")", "[": "]", "{": "}"}


def _skip_group(toks, i):
    """toks[i] is an opening bracket; return the index after its match."""
    depth = 0
    while True:
        t = toks[i].t
        if toks[i].k == "p" and t in "([{":
            depth += 1
        elif toks[i].k == "p" and t in ")]}":
            depth -= 1
            if depth == 0:
                return i + 1
        elif toks[i].k == "eof":
            raise TranslateError("unbalanced brackets")
        i += 1


def _eval_cfg(toks):
    """Evaluate the token list of a cfg(...) predicate."""
    toks = list(toks) + [Tok("eof", "", 0)]
    pos = [0]

    def pred():
        t = toks[pos[0]].t
        pos[0] += 1
        if t in ("all", "any", "not"):
            assert toks[pos[0]].t == "("
            pos[0] += 1
            vals = []
            while toks[pos[0]].t != ")":
                vals.append(pred())
                if toks[pos[0]].t == ",":
                    pos[0] += 1
            pos[0] += 1
            if t == "all":
                return all(vals)
            if t == "any":
                return any(vals)
            return not vals[0]
        if toks[pos[0]].t == "=":
            val = toks[pos[0] + 1].t.strip('"')
            pos[0] += 2
            return val in CFG.get(t, set())
        return bool(CFG.get(t, False))
    return pred()


class Item:
    def __init__(self, kind, name, start, end, attrs, header=None):
        self.kind, self.name, self.start, self.end = kind, name, start, end
        self.attrs, self.header = attrs, header
        self.children = []


def skim(toks, i, stop):
    """Split toks[i:stop] into items (attributes, kind, name, extent)."""
    items = []
    while i < stop and toks[i].k != "eof":
        attrs, keep = [], True
        while toks[i].t == "#":
            j = i + 1
            if toks[j].t == "!":
                j += 1
            end = _skip_group(toks, j)
            body = toks[j + 1:end - 1]
            if body and body[0].t == "cfg":
                keep = keep and _eval_cfg(body[2:-1])
            attrs.append(body)
            i = end
        start = i
        if toks[i].t == "pub":
            i += 1
            if toks[i].t == "(":
                i = _skip_group(toks, i)
        while toks[i].t in ("unsafe", "const", "extern", "async") and toks[i + 1].t != "=" and \
                not (toks[i].t == "const" and toks[i + 2].t == ":"):
            i += 1
            if toks[i].k == "str":
                i += 1
        kw = toks[i].t
        if kw == "fn":
            name = toks[i + 1].t
            j = i
            while toks[j].t not in ("{", ";"):
                j = _skip_group(toks, j) if toks[j].t in "([" and toks[j].k == "p" else j + 1
            end = _skip_group(toks, j) if toks[j].t == "{" else j + 1
            it = Item("fn" if toks[j].t == "{" else "fn_decl", name, start, end, attrs)
        elif kw in ("struct", "enum", "union", "trait", "mod"):
            name = toks[i + 1].t
            j = i + 2
            while toks[j].t not in ("{", ";"):
                j = _skip_group(toks, j) if toks[j].t in "([" and toks[j].k == "p" else j + 1
            end = _skip_group(toks, j) if toks[j].t == "{" else j + 1
            it = Item(kw, name, start, end, attrs)
            if kw == "trait":
                it.children = skim(toks, j + 1, end - 1)
                it.body_start = j + 1
        elif kw == "impl":
            j = i + 1
            if toks[j].t == "<":
                depth = 0
                while True:
                    depth += {"<": 1, ">": -1}.get(toks[j].t, 0)
                    j += 1
                    if depth == 0:
                        break
            hdr_start = j
            while toks[j].t != "{":
                j += 1
            hdr = toks[hdr_start:j]
            names = [t.t for t in hdr]
            if "for" in names:
                k = names.index("for")
                key = "%s for %s" % (names[0], names[k + 1])
            else:
                key = names[0]
            end = _skip_group(toks, j)
            it = Item("impl", key, start, end, attrs, header=(i, j))
            it.children = skim(toks, j + 1, end - 1)
        elif kw in ("use", "type", "const", "static", "crate"):
            name = toks[i + 1].t
            j = i
            while toks[j].t != ";":
                j = _skip_group(toks, j) if toks[j].t in "([{" and toks[j].k == "p" else j + 1
            end = j + 1
            it = Item(kw, name, start, end, attrs)
        elif kw == "macro_rules":
            j = i + 3
            end = _skip_group(toks, j)
            if toks[end].t == ";":
                end += 1
            it = Item("macro_rules", toks[i + 2].t, start, end, attrs)
        elif toks[i].k == "id" and toks[i + 1].t == "!":
            end = _skip_group(toks, i + 2)
            if toks[end].t == ";":
                end += 1
            it = Item("macro", kw, start, end, attrs)
        else:
            raise TranslateError("line %d: unexpected item start %r" % (toks[i].line, kw))
        if keep:
            items.append(it)
        i = end
    return items


# ---------------------------------------------------------------- parser
PREC = {"||": 1, "&&": 2, "==": 3, "!=": 3, "<": 3, ">": 3, "<=": 3, ">=": 3,
        "|": 4, "^": 5, "&": 6, "+": 8, "-": 8, "*": 9, "/": 9, "%": 9}
ASSIGN = ("=", "+=", "-=", "*=", "/=", "%=")


class Parser:
    def __init__(self, toks, path):
        self.toks, self.i, self.path = toks, 0, path

    # -- helpers
    def peek(self, k=0):
        return self.toks[self.i + k]

    def at(self, *ts):
        return self.peek().t in ts and self.peek().k in ("p", "id")

    def next(self):
        t = self.toks[self.i]
        self.i += 1
        return t

    def expect(self, t):
        tok = self.next()
        if tok.t != t:
            self.fail("expected %r, got %r" % (t, tok.t), tok)
        return tok

    def fail(self, msg, tok=None):
        tok = tok or self.peek()
        raise TranslateError("%s:%d: %s" % (self.path, tok.line, msg))

    def ident(self):
        tok = self.next()
        if tok.k != "id":
            self.fail("expected identifier, got %r" % tok.t, tok)
        return tok.t

    # -- types
    def type_(self):
        if self.at("&"):
            self.next()
            mut = False
            if self.at("mut"):
                self.next()
                mut = True
            return ("ref", mut, self.type_())
        if self.at("("):
            self.next()
            elems = []
            while not self.at(")"):
                elems.append(self.type_())
                if self.at(","):
                    self.next()
            self.next()
            return ("tuple", elems)
        if self.at("["):
            self.next()
            el = self.type_()
            if self.at(";"):
                self.next()
                n = self.expr()
                self.expect("]")
                return ("array", el, n)
            self.expect("]")
            return ("slice", el)
        if self.at("dyn"):
            self.next()
            return ("dyn", self.ident())
        segs = []
        while True:
            name = self.ident()
            args = []
            if self.at("<"):
                args = self.generic_args()
            segs.append((name, args))
            if self.at("::"):
                self.next()
                continue
            break
        return ("path", segs)

    def generic_args(self):
        self.expect("<")
        args = []
        while not self.at(">"):
            if self.peek().k == "num":
                args.append(("const", self.next().t))
            else:
                args.append(self.type_())
            if self.at(","):
                self.next()
        self.expect(">")
        return args

    def generics(self):
        """<const P: u8, T: Bound, ...> -> [(kind, name, type-or-None)]"""
        out = []
        if not self.at("<"):
            return out
        self.next()
        while not self.at(">"):
            if self.at("const"):
                self.next()
                name = self.ident()
                self.expect(":")
                out.append(("const", name, self.type_()))
            else:
                name = self.ident()
                if self.at(":"):
                    self.next()
                    self.bounds()
                out.append(("type", name, None))
            if self.at(","):
                self.next()
        self.next()
        return out

    def bounds(self):
        """Skip or parse trait bounds; returns ('fn', args, ret) for Fn* bounds."""
        result = None
        while True:
            if self.at("?"):
                self.next()
            name = self.ident()
            while self.at("::"):
                self.next()
                name = self.ident()
            if name in ("FnMut", "Fn", "FnOnce") and self.at("("):
                self.next()
                args = []
                while not self.at(")"):
                    args.append(self.type_())
                    if self.at(","):
                        self.next()
                self.next()
                ret = None
                if self.at("->"):
                    self.next()
                    ret = self.type_()
                result = ("fn", args, ret)
            elif self.at("<"):
                self.generic_args()
            if self.at("+"):
                self.next()
                continue
            return result

    def where_clause(self):
        out = {}
        if not self.at("where"):
            return out
        self.next()
        while not self.at("{"):
            name = self.ident()
            self.expect(":")
            b = self.bounds()
            if b:
                out[name] = b
            if self.at(","):
                self.next()
        return out

    # -- functions
    def fn(self):
        while not self.at("fn"):
            self.next()
        self.next()
        name = self.ident()
        gens = self.generics()
        self.expect("(")
        params = []
        while not self.at(")"):
            if self.at("&") and self.peek(1).t in ("self", "mut"):
                self.next()
                mut = False
                if self.at("mut"):
                    self.next()
                    mut = True
                self.expect("self")
                params.append(("self", "mref" if mut else "ref"))
            elif self.at("self") or (self.at("mut") and self.peek(1).t == "self"):
                if self.at("mut"):
                    self.next()
                self.next()
                params.append(("self", "val"))
            else:
                pat = self.pattern()
                self.expect(":")
                params.append(("param", pat, self.type_()))
            if self.at(","):
                self.next()
        self.next()
        ret = None
        if self.at("->"):
            self.next()
            ret = self.type_()
        where = self.where_clause()
        body = self.block()
        return {"name": name, "generics": gens, "params": params, "ret": ret, "where": where,
                "body": body}

    # -- patterns
    def pattern(self):
        if self.at("&"):
            self.next()
            return ("ref", self.pattern())
        if self.at("("):
            self.next()
            elems = []
            while not self.at(")"):
                elems.append(self.pattern())
                if self.at(","):
                    self.next()
            self.next()
            return ("tuple", elems)
        if self.at("_"):
            self.next()
            return ("wild",)
        if self.peek().k == "num" or (self.at("-") and self.peek(1).k == "num"):
            return ("lit", self.unary())
        mut = False
        if self.at("mut"):
            self.next()
            mut = True
        return ("ident", self.ident(), mut)

    # -- statements and blocks
    def block(self):
        self.expect("{")
        stmts, tail = [], None
        while not self.at("}"):
            if self.at(";"):
                self.next()
                continue
            while self.at("#"):  # attributes on statements
                self.next()
                self.i = _skip_group(self.toks, self.i)
            if self.at("let"):
                self.next()
                pat = self.pattern()
                ty = None
                if self.at(":"):
                    self.next()
                    ty = self.type_()
                init = None
                if self.at("="):
                    self.next()
                    init = self.expr()
                self.expect(";")
                stmts.append(("let", pat, ty, init))
                continue
            if self.at("const") and self.peek(2).t == ":":
                self.next()
                name = self.ident()
                self.expect(":")
                ty = self.type_()
                self.expect("=")
                e = self.expr()
                self.expect(";")
                stmts.append(("const", name, ty, e))
                continue
            if self.at("for"):
                self.next()
                pat = self.pattern()
                self.expect("in")
                it = self.expr(no_struct=True)
                body = self.block()
                stmts.append(("for", pat, it, body))
                continue
            e = self.expr()
            if self.at(";"):
                self.next()
                stmts.append(("expr", e))
            elif self.at("}"):
                tail = e
            elif e[0] in ("if", "match", "block"):
                stmts.append(("expr", e))
            else:
                self.fail("expected ';' after expression")
        self.next()
        return ("block", stmts, tail)

    # -- expressions
    def expr(self, no_struct=False):
        lhs = self.range_expr(no_struct)
        if self.at(*ASSIGN):
            op = self.next().t
            rhs = self.expr(no_struct)
            return ("assign", op, lhs, rhs)
        return lhs

    def range_expr(self, no_struct):
        if self.at("..", "..="):
            incl = self.next().t == "..="
            hi = None if self._ends_expr() else self.binary(0, no_struct)
            return ("range", None, hi, incl)
        lo = self.binary(0, no_struct)
        if self.at("..", "..="):
            incl = self.next().t == "..="
            hi = None if self._ends_expr() else self.binary(0, no_struct)
            return ("range", lo, hi, incl)
        return lo

    def _ends_expr(self):
        return self.at(")", "]", "}", ",", ";") or (self.at("{"))

    def binary(self, min_prec, no_struct):
        lhs = self.unary(no_struct)
        while True:
            t = self.peek()
            if t.k == "id" and t.t == "as":
                self.next()
                lhs = ("cast", lhs, self.type_())
                continue
            if t.k != "p" or t.t not in PREC or PREC[t.t] <= min_prec - 1 or PREC[t.t] < min_prec:
                return lhs
            op = self.next().t
            rhs = self.binary(PREC[op] + 1, no_struct)
            lhs = ("bin", op, lhs, rhs)

    def unary(self, no_struct=False):
        if self.at("-"):
            self.next()
            return ("unary", "-", self.unary(no_struct))
        if self.at("!"):
            self.next()
            return ("unary", "!", self.unary(no_struct))
        if self.at("&"):
            self.next()
            if self.at("mut"):
                self.next()
            return ("addr", self.unary(no_struct))
        if self.at("*"):
            self.next()
            return ("deref", self.unary(no_struct))
        e = self.postfix(self.primary(no_struct))
        # `as` binds tighter than any binary operator but looser than unary
        while self.peek().k == "id" and self.peek().t == "as":
            self.next()
            e = ("cast", e, self.type_())
        return e

    def postfix(self, e):
        while True:
            if self.at("."):
                self.next()
                if self.peek().k == "num":
                    e = ("field", e, "_" + self.next().t)
                    continue
                name = self.ident()
                turbo = []
                if self.at("::"):
                    self.next()
                    turbo = self.generic_args()
                if self.at("("):
                    e = ("mcall", e, name, turbo, self.args())
                else:
                    e = ("field", e, name)
            elif self.at("("):
                e = ("call", e, self.args())
            elif self.at("["):
                self.next()
                idx = self.expr()
                self.expect("]")
                e = ("index", e, idx)
            elif self.at("?"):
                self.fail("`?` is outside the translated subset")
            else:
                return e

    def args(self):
        self.expect("(")
        out = []
        while not self.at(")"):
            out.append(self.expr())
            if self.at(","):
                self.next()
        self.next()
        return out

    def primary(self, no_struct=False):
        t = self.peek()
        if t.k == "num":
            self.next()
            return ("num", t.t)
        if t.k == "str":
            self.next()
            return ("str", t.t)
        if t.t in ("true", "false"):
            self.next()
            return ("bool", t.t)
        if t.t == "(":
            self.next()
            elems, trailing = [], False
            while not self.at(")"):
                elems.append(self.expr())
                trailing = False
                if self.at(","):
                    self.next()
                    trailing = True
            self.next()
            if len(elems) == 1 and not trailing:
                return ("paren", elems[0])
            return ("tuple", elems)
        if t.t == "[":
            self.next()
            elems = []
            while not self.at("]"):
                elems.append(self.expr())
                if self.at(";"):
                    self.fail("[x; n] array literals are outside the translated subset")
                if self.at(","):
                    self.next()
            self.next()
            return ("array", elems)
        if t.t == "{":
            return self.block()
        if t.t == "unsafe":
            self.next()
            return self.block()
        if t.t == "if":
            return self.if_expr()
        if t.t == "match":
            self.next()
            scrut = self.expr(no_struct=True)
            self.expect("{")
            arms = []
            while not self.at("}"):
                pat = self.pattern()
                self.expect("=>")
                body = self.expr()
                arms.append((pat, body))
                if self.at(","):
                    self.next()
            self.next()
            return ("match", scrut, arms)
        if t.t in ("|", "||", "move"):
            return self.closure()
        if t.t == "return":
            self.next()
            if self._ends_expr():
                return ("return", None)
            return ("return", self.expr())
        if t.t == "break":
            self.next()
            return ("break",)
        if t.t == "continue":
            self.next()
            return ("continue",)
        if t.k == "id":
            # macro invocation
            if self.peek(1).t == "!" and self.peek(2).t in ("(", "["):
                name = self.next().t
                self.next()
                j = self.i
                end = _skip_group(self.toks, j)
                inner = self.toks[j + 1:end - 1]
                self.i = end
                return ("macro", name, inner)
            segs = []
            while True:
                name = self.ident()
                args = []
                if self.at("::") and self.peek(1).t == "<":
                    self.next()
                    args = self.generic_args()
                segs.append((name, args))
                if self.at("::") and self.peek(1).k == "id":
                    self.next()
                    continue
                break
            if self.at("{") and not no_struct and segs[-1][0][:1].isupper():
                return self.struct_lit(segs)
            return ("path", segs)
        self.fail("unexpected token %r" % t.t)

    def if_expr(self):
        self.expect("if")
        cond = self.expr(no_struct=True)
        then = self.block()
        els = None
        if self.at("else"):
            self.next()
            els = self.if_expr() if self.at("if") else self.block()
        return ("if", cond, then, els)

    def closure(self):
        if self.at("move"):
            self.next()
        params = []
        if self.at("||"):
            self.next()
        else:
            self.expect("|")
            while not self.at("|"):
                params.append(self.pattern())
                if self.at(":"):
                    self.next()
                    self.type_()
                if self.at(","):
                    self.next()
            self.next()
        if self.at("->"):
            self.next()
            self.type_()
        body = self.expr()
        return ("closure", params, body)

    def struct_lit(self, segs):
        self.expect("{")
        fields = []
        while not self.at("}"):
            name = self.ident()
            if self.at(":"):
                self.next()
                fields.append((name, self.expr()))
            else:
                fields.append((name, ("path", [(name, [])])))
            if self.at(","):
                self.next()
        self.next()
        return ("struct", segs, fields)


# ---------------------------------------------------------------- emitter
CPP_KEYWORDS = {"auto", "bool", "char", "class", "default", "delete", "double", "float", "int",
                "long", "namespace", "new", "operator", "private", "protected", "public",
                "register", "short", "signed", "sizeof", "switch", "template", "this", "throw",
                "try", "typedef", "typename", "union", "unsigned", "virtual", "void", "volatile",
                "case", "catch", "friend", "goto", "inline", "explicit", "export", "extern",
                "static", "struct", "do", "while", "and", "or", "not", "xor", "bitand", "bitor"}
PRIM = {"f32": "float", "f64": "double", "u8": "uint8_t", "u16": "uint16_t", "u32": "uint32_t",
        "u64": "uint64_t", "usize": "size_t", "i8": "int8_t", "i16": "int16_t",
        "i32": "int32_t", "i64": "int64_t", "isize": "ptrdiff_t", "bool": "bool"}
SHIM_TYPES = {"Point3", "Vector3", "Range", "Duration", "Instant", "Option", "Vec", "__m128",
              "__m128i"}
OPERATOR_TRAITS = {("Add", "add"): "operator+", ("Sub", "sub"): "operator-",
                   ("Mul", "mul"): "operator*", ("Div", "div"): "operator/",
                   ("Neg", "neg"): "operator-", ("Index", "index"): "rs_index"}
MODULE_PREFIXES = {"iter", "self", "super", "crate", "std", "math", "grid", "cmp"}
INT_SUFFIX = {"u8", "u16", "u32", "u64", "usize", "i8", "i16", "i32", "i64", "isize"}


class Ctx:
    """What the emitter knows while translating one function."""

    def __init__(self, fn_name, self_type=None, self_base=None, assoc=None, const_generics=(),
                 type_generics=(), structs=None, fn_body=None):
        self.fn_name = fn_name
        self.self_type = self_type
        self.self_base = self_base
        self.assoc = assoc or {}
        self.const_generics = set(const_generics)
        self.type_generics = set(type_generics)
        self.structs = structs or {}
        self.fn_body = fn_body
        self.scopes = [{}]
        self.counter = {}
        self.tmp = 0

    def fresh(self, name):
        n = self.counter.get(name, 0)
        self.counter[name] = n + 1
        base = name + "_" if name in CPP_KEYWORDS else name
        return base if n == 0 else "%s__%d" % (base, n)

    def bind(self, name):
        cname = self.fresh(name)
        self.scopes[-1][name] = cname
        return cname

    def lookup(self, name):
        for s in reversed(self.scopes):
            if name in s:
                return s[name]
        return None

    def push(self):
        self.scopes.append({})

    def pop(self):
        self.scopes.pop()

    def temp(self):
        self.tmp += 1
        return "__t%d" % self.tmp


class Emitter:
    def __init__(self, structs, tuple_structs, type_aliases):
        self.structs = structs              # name -> (generics, [(field, type)])
        self.tuple_structs = tuple_structs  # name -> generics
        self.type_aliases = type_aliases

    # -- types
    def ty(self, t, ctx, const_ref=True):
        k = t[0]
        if k == "ref":
            inner = self.ty(t[2], ctx)
            if t[2][0] == "dyn":
                return inner
            return ("%s&" % inner) if t[1] else ("const %s&" % inner)
        if k == "tuple":
            if not t[1]:
                return "void"
            return "std::tuple<%s>" % ", ".join(self.ty(e, ctx) for e in t[1])
        if k == "array":
            return "std::array<%s, %s>" % (self.ty(t[1], ctx), self.expr(t[2], ctx))
        if k == "slice":
            return "Slice<%s>" % self.ty(t[1], ctx)
        if k == "dyn":
            return ctx.dyn_params.setdefault(t[1], "Dyn%s" % t[1])
        if k == "const":
            return t[1]
        segs = t[1]
        if len(segs) == 2 and segs[0][0] == "Self" and segs[1][0] in ctx.assoc:
            return ctx.assoc[segs[1][0]]
        segs = [s for s in segs if s[0] not in MODULE_PREFIXES] or segs[-1:]
        if len(segs) != 1:
            raise TranslateError("type path %s outside the subset" % "::".join(s[0] for s in segs))
        name, args = segs[0]
        if name == "Self":
            return ctx.self_type
        if name in PRIM:
            return PRIM[name]
        if name in ctx.type_generics or name in ctx.const_generics:
            return name
        if name == "Vec":
            return "std::vector<%s>" % self.ty(args[0], ctx)
        if name == "Option":
            return "std::optional<%s>" % self.ty(args[0], ctx)
        if name == "String":
            raise TranslateError("String is outside the subset")
        if name in self.type_aliases:
            return name
        if args:
            return "%s<%s>" % (name, ", ".join(self.ty(a, ctx) for a in args))
        if name in self.structs and self.structs[name][0]:
            raise TranslateError("generic struct %s used without arguments" % name)
        return name

    # -- patterns
    def bind_pattern(self, pat, ctx):
        """Binds the names of `pat`; returns a C++ declarator ('x' or '[a, b]')."""
        k = pat[0]
        if k == "ref":
            return self.bind_pattern(pat[1], ctx)
        if k == "wild":
            return ctx.temp()
        if k == "ident":
            return ctx.bind(pat[1])
        if k == "tuple":
            return "[%s]" % ", ".join(self.bind_pattern(p, ctx) for p in pat[1])
        raise TranslateError("pattern %r outside the subset" % (pat,))

    # -- literals
    @staticmethod
    def num(text):
        t = text.replace("_", "")
        for suf in ("f32", "f64"):
            if t.endswith(suf) and not t.startswith("0x"):
                if suf == "f64":
                    raise TranslateError("f64 literal %s" % text)
                t = t[:-3]
                if "." not in t and "e" not in t.lower():
                    t += ".0"
                return t + "f"
        for suf in sorted(INT_SUFFIX, key=len, reverse=True):
            if t.endswith(suf) and not (t.startswith("0x") and suf in ("u8",)):
                return "%s(%s)" % (PRIM[suf], t[:-len(suf)])
        if t.startswith(("0x", "0b")):
            return t
        if "." in t or "e" in t.lower():
            return t + "f"
        return t

    # -- expressions
    def expr(self, e, ctx):
        k = e[0]
        if k == "num":
            return self.num(e[1])
        if k == "bool":
            return e[1]
        if k == "str":
            return e[1]
        if k == "paren":
            return "(%s)" % self.expr(e[1], ctx)
        if k == "path":
            return self.path(e[1], ctx)
        if k == "tuple":
            if not e[1]:
                return "void()"
            return "std::make_tuple(%s)" % ", ".join(self.expr(x, ctx) for x in e[1])
        if k == "array":
            return "rs_arr(%s)" % ", ".join(self.expr(x, ctx) for x in e[1])
        if k == "unary":
            return "(%s%s)" % (e[1], self.expr(e[2], ctx))
        if k == "addr":
            return self.expr(e[1], ctx)
        if k == "deref":
            return self.expr(e[1], ctx)
        if k == "bin":
            return "(%s %s %s)" % (self.expr(e[2], ctx), e[1], self.expr(e[3], ctx))
        if k == "cast":
            return "static_cast<%s>(%s)" % (self.ty(e[2], ctx), self.expr(e[1], ctx))
        if k == "range":
            if e[3]:
                raise TranslateError("inclusive ranges are outside the subset")
            if e[1] is None and e[2] is None:
                raise TranslateError("`..` is outside the subset")
            if e[2] is None:
                return "rs_range_from(%s)" % self.expr(e[1], ctx)
            if e[1] is None:
                raise TranslateError("`..b` is outside the subset")
            return "rs_range(%s, %s)" % (self.expr(e[1], ctx), self.expr(e[2], ctx))
        if k == "field":
            return "%s.%s" % (self.expr(e[1], ctx), e[2])
        if k == "index":
            return "rs_index(%s, %s)" % (self.expr(e[1], ctx), self.expr(e[2], ctx))
        if k == "mcall":
            if e[3]:
                raise TranslateError("turbofish on method %s" % e[2])
            args = [self.expr(e[1], ctx)] + [self.expr(a, ctx) for a in e[4]]
            return "m_%s(%s)" % (e[2], ", ".join(args))
        if k == "call":
            return self.call(e, ctx)
        if k == "struct":
            return self.struct_lit(e, ctx)
        if k == "block":
            return self.block_value(e, ctx)
        if k == "if":
            if e[3] is None:
                raise TranslateError("`if` without `else` used as a value")
            return "(%s ? %s : %s)" % (self.expr(e[1], ctx), self.block_value(e[2], ctx),
                                       self.block_value(e[3], ctx) if e[3][0] == "block"
                                       else self.expr(e[3], ctx))
        if k == "match":
            return self.match_value(e, ctx)
        if k == "closure":
            return self.closure(e, ctx)
        if k == "macro":
            return self.macro(e, ctx)
        if k == "assign":
            return "%s %s %s" % (self.expr(e[2], ctx), e[1], self.expr(e[3], ctx))
        raise TranslateError("expression %s outside the subset" % k)

    def path(self, segs, ctx, calling=False):
        names = [s[0] for s in segs]
        if len(segs) == 1:
            name = names[0]
            local = ctx.lookup(name)
            if local is not None:
                return local
            if name == "self":
                return "self"
            if name == "None":
                return "std::nullopt"
            if name in ctx.const_generics:
                return name
            targs = segs[0][1]
            if targs:
                return "%s<%s>" % (name, ", ".join(self.ty(a, ctx) for a in targs))
            return name
        while len(segs) > 2 and segs[0][0] in MODULE_PREFIXES:
            segs = segs[1:]
        if len(segs) == 2 and segs[0][0] in MODULE_PREFIXES:
            return self.path(segs[1:], ctx, calling)
        if len(segs) != 2:
            raise TranslateError("path %s outside the subset" % "::".join(names))
        (tname, targs), (fname, fargs) = segs
        if tname == "Self":
            tname = ctx.self_base
        if tname in ctx.type_generics:
            return "assoc__%s<%s>" % (fname, tname)
        out = "%s__%s" % (tname, fname)
        if fargs or targs:
            out += "<%s>" % ", ".join(self.ty(a, ctx) for a in (targs + fargs))
        return out

    def call(self, e, ctx):
        callee, args = e[1], e[2]
        a = [self.expr(x, ctx) for x in args]
        if callee[0] == "path":
            segs = callee[1]
            last = segs[-1][0]
            # tuple-struct constructor: Self(x) / Vec3(x)
            name = ctx.self_base if last == "Self" and len(segs) == 1 else last
            if len(segs) == 1 and name in self.tuple_structs and ctx.lookup(last) is None:
                tname = ctx.self_type if last == "Self" else name
                return "%s{%s}" % (tname, ", ".join(a))
            if len(segs) == 1 and last == "Some":
                return "Some(%s)" % a[0]
            if len(segs) == 2 and segs[0][0] == "Vec":
                raise TranslateError("Vec::%s needs a type; only `let v = Vec::..` is supported"
                                     % last)
            return "%s(%s)" % (self.path(segs, ctx, calling=True), ", ".join(a))
        return "%s(%s)" % (self.expr(callee, ctx), ", ".join(a))

    def struct_lit(self, e, ctx):
        segs, fields = e[1], e[2]
        name = segs[-1][0]
        if name == "Self" or name == ctx.self_base:
            tname = ctx.self_type
        else:
            if name not in self.structs:
                raise TranslateError("struct literal of unknown type %s" % name)
            if self.structs[name][0]:
                raise TranslateError("generic struct literal %s outside its impl" % name)
            tname = name
        tmp = ctx.temp()
        parts = ["%s %s{};" % (tname, tmp)]
        for f, x in fields:
            parts.append("%s.%s = %s;" % (tmp, f, self.expr(x, ctx)))
        parts.append("%s;" % tmp)
        return "({ %s })" % " ".join(parts)

    def closure(self, e, ctx):
        params, body = e[1], e[2]
        ctx.push()
        decls, pro = [], []
        for n, p in enumerate(params):
            base = p[1] if p[0] == "ref" else p
            if base[0] == "ident":
                decls.append("auto %s" % ctx.bind(base[1]))
            else:
                arg = "__a%d_%d" % (ctx.tmp, n)
                ctx.tmp += 1
                decls.append("auto %s" % arg)
                pro.append("auto %s = %s;" % (self.bind_pattern(base, ctx), arg))
        if body[0] == "block":
            inner = self.block_lines(body, ctx, "return", push=True)
        else:
            inner = ["return %s;" % self.expr(body, ctx)]
        ctx.pop()
        return "[&](%s) { %s }" % (", ".join(decls), " ".join(pro + inner))

    def macro(self, e, ctx):
        name, toks = e[1], e[2]
        if name in ("trace", "debug", "info", "warn", "debug_assert", "debug_assert_eq"):
            return "(void)0"
        if name == "assert":
            sub = Parser(toks + [Tok("eof", "", 0)], "assert!")
            cond = sub.expr()
            return "rs_assert(%s, \"%s\")" % (self.expr(cond, ctx), ctx.fn_name)
        raise TranslateError("macro %s! outside the subset" % name)

    def match_value(self, e, ctx):
        scrut = self.expr(e[1], ctx)
        out = None
        for pat, body in reversed(e[2]):
            val = self.expr(body, ctx) if body[0] != "block" else self.block_value(body, ctx)
            if pat[0] == "wild":
                out = val
            elif pat[0] == "lit":
                if out is None:
                    raise TranslateError("match without a final `_` arm")
                out = "((%s) == (%s) ? %s : %s)" % (scrut, self.expr(pat[1], ctx), val, out)
            else:
                raise TranslateError("match pattern outside the subset")
        return out

    # -- blocks and statements
    def block_value(self, b, ctx):
        lines = self.block_lines(b, ctx, "value", push=True)
        return "({ %s })" % " ".join(lines)

    def block_lines(self, b, ctx, mode, push=False):
        """mode: 'stmt' (the tail's value is dropped), 'value' (the tail is the
        block's value: the last statement of a statement expression) or
        'return' (the tail is returned)."""
        if push:
            ctx.push()
        lines = []
        for s in b[1]:
            lines += self.stmt(s, ctx)
        tail = b[2]
        if tail is not None:
            if mode == "return":
                lines += self.tail_return(tail, ctx)
            elif mode == "value":
                lines.append("%s;" % self.expr(tail, ctx))
            else:
                lines += self.stmt(("expr", tail), ctx)
        if push:
            ctx.pop()
        return lines

    def tail_return(self, e, ctx):
        k = e[0]
        if k == "block":
            return ["{"] + self.block_lines(e, ctx, "return", push=True) + ["}"]
        if k == "if" and e[3] is not None:
            out = ["if (%s) {" % self.expr(e[1], ctx)]
            out += self.block_lines(e[2], ctx, "return", push=True)
            out.append("} else {")
            out += (self.block_lines(e[3], ctx, "return", push=True) if e[3][0] == "block"
                    else self.tail_return(e[3], ctx))
            out.append("}")
            return out
        if k == "match":
            scrut = e[1]
            const = scrut[0] == "path" and len(scrut[1]) == 1 and \
                scrut[1][0][0] in ctx.const_generics
            sv = self.expr(scrut, ctx)
            out = []
            if not const:
                tmp = ctx.temp()
                out.append("{ auto %s = %s;" % (tmp, sv))
                sv = tmp
            first = True
            for pat, body in e[2]:
                ret = (self.tail_return(body, ctx) if body[0] in ("block", "if", "match")
                       else ["return %s;" % self.expr(body, ctx)])
                if pat[0] == "wild":
                    out += (["{"] if first else ["else {"]) + ret + ["}"]
                    break
                if pat[0] != "lit":
                    raise TranslateError("match pattern outside the subset")
                kw = "if constexpr" if const else "if"
                out.append("%s%s ((%s) == (%s)) {" % ("" if first else "else ", kw, sv,
                                                      self.expr(pat[1], ctx)))
                out += ret + ["}"]
                first = False
            if not const:
                out.append("}")
            return out
        if k == "return":
            return self.stmt(("expr", e), ctx)
        val = self.expr(e, ctx)
        obs = getattr(ctx, "observe", False)
        if obs:
            tmp = ctx.temp()
            return ["auto %s = %s;" % (tmp, val), "rs_observe(%s);" % tmp, "return %s;" % tmp]
        return ["return %s;" % val]

    def vec_type(self, name, ctx):
        """Element type of `let name = Vec::new()`, from the struct literal that
        takes `name` as a field later in the same function."""
        found = []

        def walk(node):
            if isinstance(node, tuple):
                if node and node[0] == "struct":
                    sname = node[1][-1][0]
                    if sname == "Self":
                        sname = ctx.self_base
                    for f, x in node[2]:
                        if x == ("path", [(name, [])]) and sname in self.structs:
                            for fname, fty in self.structs[sname][1]:
                                if fname == f:
                                    found.append(fty)
                for c in node:
                    walk(c)
            elif isinstance(node, list):
                for c in node:
                    walk(c)
        walk(ctx.fn_body)
        if not found:
            raise TranslateError("cannot find the element type of Vec `%s`" % name)
        return self.ty(found[0], ctx)

    def stmt(self, s, ctx):
        k = s[0]
        if k == "let":
            pat, ty, init = s[1], s[2], s[3]
            if init is None:
                raise TranslateError("`let` without initialiser")
            if init[0] == "call" and init[1][0] == "path" and len(init[1][1]) == 2 and \
                    init[1][1][0][0] == "Vec":
                if pat[0] != "ident":
                    raise TranslateError("Vec bound to a pattern")
                vt = self.vec_type(pat[1], ctx)
                fn = init[1][1][1][0]
                args = ", ".join(self.expr(a, ctx) for a in init[2])
                decl = ctx.bind(pat[1])
                return ["auto %s = Vec__%s<%s>(%s);" % (decl, fn, vt, args)]
            val = self.expr(init, ctx)
            decl = self.bind_pattern(pat, ctx)
            if ty is not None and pat[0] == "ident":
                return ["%s %s = %s;" % (self.ty(ty, ctx), decl, val)]
            return ["auto %s = %s;" % (decl, val)]
        if k == "const":
            name, ty, e = s[1], s[2], s[3]
            if e[0] == "array" and ty[0] == "array":
                el = self.ty(ty[1], ctx)
                val = "rs_arr_as<%s>(%s)" % (el, ", ".join(self.expr(x, ctx) for x in e[1]))
            else:
                val = self.expr(e, ctx)
            return ["const %s %s = %s;" % (self.ty(ty, ctx), ctx.bind(name), val)]
        if k == "for":
            pat, it, body = s[1], s[2], s[3]
            src = self.expr(it, ctx)
            var = "__it%d" % ctx.tmp
            ctx.tmp += 1
            ctx.push()
            decl = self.bind_pattern(pat, ctx)
            lines = ["for (auto&& %s : rs_iterable(%s)) {" % (var, src),
                     "auto %s = %s;" % (decl, var)]
            lines += self.block_lines(body, ctx, "stmt", push=True)
            ctx.pop()
            lines.append("}")
            return lines
        if k == "expr":
            e = s[1]
            if e[0] == "if":
                out = ["if (%s) {" % self.expr(e[1], ctx)]
                out += self.block_lines(e[2], ctx, "stmt", push=True)
                out.append("}")
                if e[3] is not None:
                    out.append("else")
                    if e[3][0] == "block":
                        out += ["{"] + self.block_lines(e[3], ctx, "stmt", push=True) + ["}"]
                    else:
                        out += ["{"] + self.stmt(("expr", e[3]), ctx) + ["}"]
                return out
            if e[0] == "block":
                return ["{"] + self.block_lines(e, ctx, "stmt", push=True) + ["}"]
            if e[0] == "return":
                if e[1] is None:
                    return ["return;"]
                return ["return %s;" % self.expr(e[1], ctx)]
            if e[0] == "break":
                return ["break;"]
            if e[0] == "continue":
                return ["continue;"]
            return ["%s;" % self.expr(e, ctx)]
        raise TranslateError("statement %s outside the subset" % k)

    # -- functions
    def function(self, f, ctx, cname, self_param_type=None, template_prefix=None):
        ctx.dyn_params = {}
        ctx.fn_body = f["body"]
        params = []
        pro = []
        for p in f["params"]:
            if p[0] == "self":
                mode = p[1]
                st = self_param_type or ctx.self_type
                params.append({"val": "%s self", "ref": "const %s& self",
                               "mref": "%s& self"}[mode] % st)
                continue
            pat, pty = p[1], p[2]
            cty = self.ty(pty, ctx)
            if pat[0] == "ident":
                params.append("%s %s" % (cty, ctx.bind(pat[1])))
            else:
                arg = ctx.temp()
                params.append("%s %s" % (cty, arg))
                pro.append("auto %s = %s;" % (self.bind_pattern(pat, ctx), arg))
        ret = "void" if f["ret"] is None else self.ty(f["ret"], ctx)
        body = pro + self.block_lines(f["body"], ctx, "return" if f["ret"] else "stmt")
        tparams = list(template_prefix or [])
        tparams += ["class %s" % v for v in ctx.dyn_params.values()]
        # default template arguments go on the prototype only
        nodef = [t.split(" = ")[0] for t in tparams]
        head = ("template <%s>\n" % ", ".join(tparams)) if tparams else "inline "
        dhead = ("template <%s>\n" % ", ".join(nodef)) if tparams else "inline "
        tail = "%s %s(%s)" % (ret, cname, ", ".join(params))
        return head + tail + ";", dhead + tail + " {\n    " + "\n    ".join(body) + "\n}\n"


def _generic_decls(gens, ctx_types):
    out = []
    for kind, name, ty in gens:
        if kind == "const":
            out.append("%s %s" % (PRIM[ty[1][0][0]], name))
        else:
            out.append("class %s" % name)
    return out


def translate(root, items=None, observe=None):
    """Translated C++ text of `items` (default ITEMS) under the source tree
    `root`; `observe` (default OBSERVE_RETURNS) names the (type, function)
    pairs whose returned value goes through rs_observe."""
    items = ITEMS if items is None else items
    observe = OBSERVE_RETURNS if observe is None else observe
    files = {}
    for path, _ in items:
        if path not in files:
            with open(os.path.join(root, path)) as f:
                text = f.read()
            toks = lex(text, path)
            files[path] = (toks, skim(toks, 0, len(toks) - 1))

    def find(path, kind, name):
        toks, items = files[path]
        hits = [it for it in items if it.kind == kind and it.name == name]
        if not hits:
            raise TranslateError("%s: no %s %s" % (path, kind, name))
        return toks, hits

    # structs and aliases first: the emitter needs their fields
    structs, tuple_structs, aliases = {}, {}, {}
    struct_text = []
    for path, sel in items:
        if sel[0] == "type":
            toks, hits = find(path, "type", sel[1])
            p = Parser(toks, path)
            p.i = hits[0].start
            while not p.at("type"):
                p.next()
            p.next()
            name = p.ident()
            p.expect("=")
            aliases[name] = p.type_()
        if sel[0] != "struct":
            continue
        toks, hits = find(path, "struct", sel[1])
        p = Parser(toks, path)
        p.i = hits[0].start
        while not p.at("struct"):
            p.next()
        p.next()
        name = p.ident()
        gens = p.generics()
        if p.at("("):
            p.next()
            fields = []
            n = 0
            while not p.at(")"):
                fields.append(("_%d" % n, p.type_()))
                n += 1
                if p.at(","):
                    p.next()
            tuple_structs[name] = gens
        else:
            p.expect("{")
            fields = []
            while not p.at("}"):
                while p.at("#"):
                    p.next()
                    p.i = _skip_group(toks, p.i)
                if p.at("pub"):
                    p.next()
                    if p.at("("):
                        p.i = _skip_group(toks, p.i)
                fname = p.ident()
                p.expect(":")
                fields.append((fname, p.type_()))
                if p.at(","):
                    p.next()
        structs[name] = (gens, fields)

    em = Emitter(structs, tuple_structs, aliases)
    base = Ctx("")
    base.dyn_params = {}
    for name, t in aliases.items():
        struct_text.append("using %s = %s;" % (name, em.ty(t, base)))
    for path, sel in items:
        if sel[0] != "struct":
            continue
        gens, fields = structs[sel[1]]
        ctx = Ctx("", const_generics=[g[1] for g in gens if g[0] == "const"],
                  type_generics=[g[1] for g in gens if g[0] == "type"])
        ctx.dyn_params = {}
        tmpl = _generic_decls(gens, ctx)
        head = ("template <%s>\n" % ", ".join(tmpl)) if tmpl else ""
        body = "".join("    %s %s;\n" % (em.ty(t, ctx), f) for f, t in fields)
        struct_text.append("%sstruct %s {\n%s};" % (head, sel[1], body))

    protos, defs = [], []
    for path, sel in items:
        if sel[0] in ("struct", "type"):
            continue
        if sel[0] == "fn":
            toks, hits = find(path, "fn", sel[1])
            p = Parser(toks, path)
            p.i = hits[0].start
            f = p.fn()
            ctx = Ctx(f["name"], const_generics=[g[1] for g in f["generics"] if g[0] == "const"],
                      type_generics=[g[1] for g in f["generics"] if g[0] == "type"],
                      structs=structs)
            pr, d = em.function(f, ctx, f["name"],
                                template_prefix=_generic_decls(f["generics"], ctx))
            protos.append(pr)
            defs.append(d)
            continue
        if sel[0] == "trait_default":
            toks, hits = find(path, "trait", sel[1])
            meth = [c for c in hits[0].children if c.kind == "fn" and c.name == sel[2]]
            if not meth:
                raise TranslateError("%s: trait %s has no default %s" % (path, sel[1], sel[2]))
            p = Parser(toks, path)
            p.i = meth[0].start
            f = p.fn()
            ctx = Ctx(f["name"], self_type="SelfT", self_base="SelfT", type_generics=["SelfT"],
                      structs=structs)
            pr, d = em.function(f, ctx, "m_" + f["name"], template_prefix=["class SelfT"])
            protos.append(pr)
            defs.append(d)
            continue
        # impl blocks
        _, key, methods = sel
        toks, hits = find(path, "impl", key)
        found = set()
        for it in hits:
            p = Parser(toks, path)
            p.i = it.header[0] + 1
            igens = p.generics()
            hdr_types = []
            trait = None
            # header: [Trait<..> for] Type<..>
            save = p.i
            t1 = p.type_()
            if p.at("for"):
                p.next()
                trait = t1[1][-1][0]
                self_t = p.type_()
            else:
                self_t = t1
            ictx_consts = [g[1] for g in igens if g[0] == "const"]
            ictx_types = [g[1] for g in igens if g[0] == "type"]
            tmp_ctx = Ctx("", const_generics=ictx_consts, type_generics=ictx_types)
            tmp_ctx.dyn_params = {}
            self_cpp = em.ty(self_t, tmp_ctx)
            self_base = self_t[1][-1][0] if self_t[0] == "path" else self_cpp
            assoc = {}
            for c in it.children:
                if c.kind == "type":
                    q = Parser(toks, path)
                    q.i = c.start
                    while not q.at("type"):
                        q.next()
                    q.next()
                    aname = q.ident()
                    q.expect("=")
                    assoc[aname] = q.type_()
            for c in it.children:
                if c.kind != "fn" or (methods is not None and c.name not in methods):
                    continue
                found.add(c.name)
                q = Parser(toks, path)
                q.i = c.start
                f = q.fn()
                fn_consts = [g[1] for g in f["generics"] if g[0] == "const"]
                fn_types = [g[1] for g in f["generics"] if g[0] == "type"]
                ctx = Ctx(f["name"], self_type=self_cpp, self_base=self_base,
                          const_generics=ictx_consts + fn_consts,
                          type_generics=ictx_types + fn_types, structs=structs)
                ctx.dyn_params = {}
                ctx.assoc = {a: em.ty(t, ctx) for a, t in assoc.items()}
                has_self = any(pp[0] == "self" for pp in f["params"])
                ctx.observe = (self_base, f["name"]) in observe
                if trait and (trait, f["name"]) in OPERATOR_TRAITS:
                    cname = OPERATOR_TRAITS[(trait, f["name"])]
                elif has_self:
                    cname = "m_" + f["name"]
                else:
                    cname = "%s__%s" % (self_base, f["name"])
                tmpl = _generic_decls(f["generics"], ctx)
                if has_self:
                    tmpl = _generic_decls(igens, ctx) + tmpl
                else:
                    # impl generics of an associated fn come after its own, each
                    # defaulted from a `where F: FnMut(..) -> T` bound
                    for kind, gname, gty in igens:
                        src = [(fname, b) for fname, b in f["where"].items()
                               if b[0] == "fn" and b[2] is not None and b[2][0] == "path"
                               and b[2][1][0][0] == gname]
                        if src:
                            fname, b = src[0]
                            args = ", ".join([fname + "&"] + [em.ty(a, ctx) for a in b[1]])
                            tmpl.append("class %s = std::invoke_result_t<%s>" % (gname, args))
                        elif kind == "const":
                            tmpl.insert(0, "%s %s" % (PRIM[gty[1][0][0]], gname))
                        else:
                            raise TranslateError("cannot place generic %s of %s::%s"
                                                 % (gname, self_base, f["name"]))
                pr, d = em.function(f, ctx, cname, template_prefix=tmpl)
                protos.append(pr)
                defs.append(d)
        if methods is not None and set(methods) - found:
            raise TranslateError("%s: impl %s lacks %s" % (path, key, sorted(set(methods) - found)))

    text = "\n".join(struct_text) + "\n\n" + "\n".join(protos) + "\n\n" + "\n".join(defs)
    if re.search(r"\bdouble\b", text):
        raise TranslateError("the translated items use f64; float literals would be ambiguous")
    return text


WRAPPER = r"""
// ---- C entry points (written by oracle/rust_build.py, not translated) ----
using namespace rsref;

extern "C" {
typedef struct {
    int32_t kind;       /* 0 Mandelbulb<power>, 1 Sphere */
    int32_t power;
    uint64_t max_iters;
    float bailout;
    float center[3];
    float radius;
} rustref_shape;

enum { RR_OK = 0, RR_ASSERT = 1, RR_CAPACITY = 2, RR_LERP = 3, RR_INDEX = 4, RR_EINVAL = 5 };
}

template <class F>
static int with_shape(const rustref_shape* s, F&& f) {
    try {
        if (s->kind == 1) {
            auto sh = Sphere__new(Point3<float>{s->center[0], s->center[1], s->center[2]}, s->radius);
            return f(sh);
        }
        switch (s->power) {
%(cases)s
        default: return RR_EINVAL;
        }
    } catch (const Panic& p) {
        return std::strcmp(p.where, "lerp") == 0 ? RR_LERP : RR_ASSERT;
    } catch (const std::out_of_range&) {
        return RR_INDEX;
    }
}

extern "C" int rustref_de(const rustref_shape* s, const float* xyz, uint64_t n, float* out) {
    return with_shape(s, [&](const auto& sh) {
        for (uint64_t i = 0; i < n; ++i)
            out[i] = m_min_distance_from(sh, Point3<float>{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]});
        return (int)RR_OK;
    });
}

extern "C" int rustref_contains(const rustref_shape* s, const float* xyz, uint64_t n, uint8_t* out) {
    return with_shape(s, [&](const auto& sh) {
        for (uint64_t i = 0; i < n; ++i)
            out[i] = m_contains(sh, Point3<float>{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]}) ? 1 : 0;
        return (int)RR_OK;
    });
}

extern "C" int rustref_generate_for_box(const rustref_shape* s, const float span[6], uint32_t res,
                                        float* vertices7, uint64_t vcap, uint32_t* indices,
                                        uint64_t icap, uint64_t* nv, uint64_t* ni, float* dists,
                                        uint32_t* points) {
    observed_f32.clear();
    observed_u32.clear();
    int rc = with_shape(s, [&](const auto& sh) {
        Span sp{Point3<float>{span[0], span[1], span[2]}, Point3<float>{span[3], span[4], span[5]}};
        auto out = MeshBuffer__generate_for_box(sp, sh, res);
        const MeshBuffer& mb = std::get<0>(out);
        *nv = mb.vertices.size();
        *ni = mb.indices.size();
        if (mb.vertices.size() > vcap || mb.indices.size() > icap) return (int)RR_CAPACITY;
        for (size_t i = 0; i < mb.vertices.size(); ++i) {
            const Vertex& v = mb.vertices[i];
            float* o = vertices7 + 7 * i;
            o[0] = v.position[0]; o[1] = v.position[1]; o[2] = v.position[2];
            o[3] = v.normal[0]; o[4] = v.normal[1]; o[5] = v.normal[2];
            o[6] = v.distance_from_surface;
        }
        std::copy(mb.indices.begin(), mb.indices.end(), indices);
        return (int)RR_OK;
    });
    // the tables of step 1 and step 2, also when the mesher panicked later on
    if (dists && observed_f32.size() == (size_t)(res + 1) * (res + 1) * (res + 1))
        std::copy(observed_f32.begin(), observed_f32.end(), dists);
    if (points && observed_u32.size() == (size_t)res * res * res)
        std::copy(observed_u32.begin(), observed_u32.end(), points);
    return rc;
}
"""


def _cases():
    return "\n".join("        case %d: { auto sh = Mandelbulb__new<%d>(s->max_iters, s->bailout); "
                     "return f(sh); }" % (p, p) for p in POWERS)


def compile_cpp(src: str, lib: str):
    """Compile translated text (with its C entry points) into `lib`."""
    os.makedirs(os.path.dirname(lib), exist_ok=True)
    cpp = lib[:-3] + ".cpp" if lib.endswith(".so") else lib + ".cpp"
    with open(cpp, "w") as f:
        f.write(src)
    tmp = lib + ".tmp%d" % os.getpid()
    subprocess.run(["g++", *CXXFLAGS, "-I", HERE, cpp, "-o", tmp, "-lm"], check=True)
    os.replace(tmp, lib)
    return lib


def build(force: bool = False):
    """Translate, wrap and compile; returns the library path, or None when the
    reference tree is not available (an earlier build is then kept)."""
    if not available():
        return LIB if os.path.exists(LIB) else None
    root = reference_root()
    text = translate(root)
    src = ('// Translated by oracle/rust_build.py from the cantucci source tree.\n'
           '#include "rust_shim.h"\n#include <algorithm>\n#include <stdexcept>\n\n'
           'namespace rsref {\n' + text + '\n}  // namespace rsref\n' + WRAPPER % {"cases": _cases()})
    os.makedirs(OUT_DIR, exist_ok=True)
    cpp = os.path.join(OUT_DIR, "rust_ref.cpp")
    changed = force or not os.path.exists(LIB) or not os.path.exists(cpp) or open(cpp).read() != src
    if not changed and os.path.getmtime(LIB) >= max(os.path.getmtime(SHIM),
                                                    os.path.getmtime(__file__)):
        return LIB
    with open(cpp, "w") as f:
        f.write(src)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.run(["g++", *CXXFLAGS, "-I", HERE, cpp, "-o", tmp, "-lm"], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    if not available():
        sys.exit("set CANTUCCI_REFERENCE to the cantucci source tree")
    print(build(force="--force" in sys.argv))
