"""Translate the reference's WGSL compute shaders into C++ (test infrastructure).

The output reads almost token for token like the shader; oracle/wgsl/prelude.h
gives it WGSL's meaning (binary32 f32 with single roundings, WGSL conversions
and builtins, storage buffers and the storage texture the harness binds).
Only the WGSL subset that src/compute.wgsl and src/display.wgsl use is
handled, and anything else is rejected:

  const NAME: T = EXPR;          -> static const T NAME = EXPR;
  struct S { f: T, ... };        -> struct S { T f; ... };
  @group @binding var<storage, read_write> NAME: array<T>;
                                 -> static Buffer<T> NAME;
  var<uniform> NAME: T;          -> static T NAME;
  var NAME: texture_storage_2d<rgba8unorm, write>;
                                 -> static StorageTexRGBA8 NAME;
  @compute ... fn NAME(@builtin(...) p: T) { ... }
  fn NAME(p: T, ...) -> R { ... } -> static R NAME(T p, ...) { ... }
  let NAME = EXPR;               -> const auto NAME = value(EXPR);
  var NAME = EXPR;               -> auto NAME = value(EXPR);
  var NAME: T = EXPR;            -> T NAME = EXPR;
  var NAME: T;                   -> T NAME{};  (WGSL's zero value)
  vec2<f32|i32|u32>/vec3<u32>/vec4<f32>
                                 -> vec2f / vec2i / vec2u / vec3u / vec4f
  i32(e), u32(e), f32(e)         -> to_i32(e), to_u32(e), to_f32(e)
  arrayLength(&b)                -> arrayLength(b)
  float literal                  -> f32(<the literal rounded to binary32>)

A parenthesised expression of float literals only (the shader's
`(2.0 * 3.14159265359)`) is an abstract-float constant expression in WGSL:
it is evaluated here in binary64 (Python floats) and rounded to binary32
once, as WGSL concretises it.  The entry point `main` becomes `wgsl_main`.

Usage: python translate.py <compute.wgsl> <out.inc>
"""
import re
import struct
import sys

TOKEN = re.compile(r"""
    (?P<ws>\s+)
  | (?P<comment>//[^\n]*)
  | (?P<attr>@[A-Za-z_]\w*)
  | (?P<num>(\d+\.\d*|\.\d+|\d+)([eE][+-]?\d+)?[uif]?)
  | (?P<id>[A-Za-z_]\w*)
  | (?P<op>->|\+=|-=|\*=|/=|<=|>=|==|!=|&&|\|\||\+\+|--|[-+*/%<>=!&|^~?:;,.(){}\[\]])
""", re.VERBOSE)


def tokenize(src):
    out, pos = [], 0
    while pos < len(src):
        m = TOKEN.match(src, pos)
        if not m:
            raise SyntaxError(f"unexpected text at {pos}: {src[pos:pos + 30]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind in ("ws", "comment"):
            continue
        out.append((kind, m.group(kind)))
    return out


def is_float_literal(tok):
    k, v = tok
    return k == "num" and (("." in v) or ("e" in v.lower() and not v.endswith(("u", "i"))) or v.endswith("f"))


def f32_literal(value):
    bits = struct.unpack("<I", struct.pack("<f", value))[0]
    f = struct.unpack("<f", struct.pack("<I", bits))[0]
    return f"f32({float(f).hex()}f)"


def fold_products(toks):
    """Fold runs 'lit * lit ...' / 'lit / lit ...' of float literals that no
    other multiplicative operator touches (in `a + 2.0 * 3.1` the product is
    an abstract-float constant expression; in `a * 2.0 * 3.1` it is not)."""
    out = []
    i = 0
    while i < len(toks):
        if is_float_literal(toks[i]) and not (out and out[-1][0] == "op" and out[-1][1] in ("*", "/", "%")):
            j = i
            parts = [toks[i][1].rstrip("f")]
            while (j + 2 < len(toks) and toks[j + 1][0] == "op" and toks[j + 1][1] in ("*", "/")
                   and is_float_literal(toks[j + 2])):
                parts += [toks[j + 1][1], toks[j + 2][1].rstrip("f")]
                j += 2
            after = toks[j + 1] if j + 1 < len(toks) else ("op", ";")
            if len(parts) >= 3 and not (after[0] == "op" and after[1] in ("*", "/", "%")):
                value = eval("".join(parts), {"__builtins__": {}}, {})  # binary64 arithmetic
                out.append(("num", repr(float(value))))
                i = j + 1
                continue
        out.append(toks[i])
        i += 1
    return out


def fold_constants(toks):
    """Replace '( lit op lit ... )' of float literals by one abstract literal."""
    toks = fold_products(toks)
    out = []
    i = 0
    while i < len(toks):
        if toks[i] == ("op", "("):
            j = i + 1
            parts = []
            ok = True
            while j < len(toks) and toks[j] != ("op", ")"):
                k, v = toks[j]
                if is_float_literal(toks[j]):
                    parts.append(v.rstrip("f"))
                elif k == "op" and v in "+-*/" and len(v) == 1:
                    parts.append(v)
                else:
                    ok = False
                    break
                j += 1
            if ok and j < len(toks) and len(parts) >= 3 and len(parts) % 2 == 1:
                value = eval("".join(parts), {"__builtins__": {}}, {})  # binary64 arithmetic
                out.append(("num", repr(float(value))))
                i = j + 1
                continue
        out.append(toks[i])
        i += 1
    return out


TYPES = {("vec2", "f32"): "vec2f", ("vec2", "i32"): "vec2i", ("vec2", "u32"): "vec2u", ("vec3", "u32"): "vec3u",
         ("vec4", "f32"): "vec4f"}


def parse_type(toks, i):
    """Type starting at toks[i]; returns (c++ type, next index)."""
    k, v = toks[i]
    if v in ("vec2", "vec3", "vec4"):
        assert toks[i + 1] == ("op", "<") and toks[i + 3] == ("op", ">"), toks[i:i + 4]
        t = TYPES.get((v, toks[i + 2][1]))
        if t is None:
            raise SyntaxError(f"unsupported type {v}<{toks[i + 2][1]}>")
        return t, i + 4
    if v == "array":
        assert toks[i + 1] == ("op", "<")
        inner, j = parse_type(toks, i + 2)
        assert toks[j] == ("op", ">")
        return f"Buffer<{inner}>", j + 1
    if v == "texture_storage_2d":
        fmt = [t[1] for t in toks[i + 1:i + 6]]
        if fmt != ["<", "rgba8unorm", ",", "write", ">"]:
            raise SyntaxError(f"unsupported storage texture {fmt}")
        return "StorageTexRGBA8", i + 6
    if k == "id":
        return v, i + 1
    raise SyntaxError(f"not a type: {toks[i]}")


def skip_attrs(toks, i):
    while toks[i][0] == "attr":
        i += 1
        if toks[i] == ("op", "("):
            depth = 0
            while True:
                if toks[i] == ("op", "("):
                    depth += 1
                elif toks[i] == ("op", ")"):
                    depth -= 1
                i += 1
                if depth == 0:
                    break
    return i


def expr_tokens(toks, i, stop=(";",)):
    """Tokens of an expression up to a top-level stop token; returns (list, index of stop)."""
    depth = 0
    out = []
    while True:
        k, v = toks[i]
        if depth == 0 and k == "op" and v in stop:
            return out, i
        if v in ("(", "[", "{"):
            depth += 1
        elif v in (")", "]", "}"):
            depth -= 1
        out.append(toks[i])
        i += 1


def emit_expr(toks):
    out = []
    i = 0
    while i < len(toks):
        k, v = toks[i]
        if k == "id" and v in ("vec2", "vec3", "vec4") and i + 1 < len(toks) and toks[i + 1] == ("op", "<"):
            t, i = parse_type(toks, i)
            # constructor call: vecNx(a, b, ...) -> vecNx{a, b, ...}
            assert toks[i] == ("op", "(")
            args, j = expr_tokens(toks, i + 1, stop=(")",))
            out.append(t + "{" + emit_expr(args) + "}")
            i = j + 1
            continue
        if k == "id" and v in ("i32", "u32", "f32") and i + 1 < len(toks) and toks[i + 1] == ("op", "("):
            out.append("to_" + v)
            i += 1
            continue
        if k == "id" and v == "arrayLength":
            out.append(v)
            i += 1
            if toks[i] == ("op", "(") and toks[i + 1] == ("op", "&"):
                out.append("(")
                i += 2
            continue
        if k == "num":
            if is_float_literal(toks[i]):
                out.append(f32_literal(float(v.rstrip("f"))))
            elif v.endswith("i"):
                out.append(v[:-1])
            else:
                out.append(v)
            i += 1
            continue
        if k == "attr":
            raise SyntaxError(f"attribute inside an expression: {v}")
        out.append(v)
        i += 1
    s = " ".join(out)
    return re.sub(r"\s*([.(\[\]),])\s*", lambda m: m.group(1) + (" " if m.group(1) == "," else ""), s)


def translate_body(toks, i):
    """Translate a { ... } block starting at toks[i] == '{'; returns (text, next index)."""
    assert toks[i] == ("op", "{")
    out = ["{"]
    i += 1
    while toks[i] != ("op", "}"):
        k, v = toks[i]
        if v in ("let", "var") and k == "id":
            name = toks[i + 1][1]
            j = i + 2
            ctype = None
            if toks[j] == ("op", ":"):
                ctype, j = parse_type(toks, j + 1)
            if v == "var" and ctype and toks[j] == ("op", ";"):
                out.append(f"{ctype} {name}{{}};")
                i = j + 1
                continue
            assert toks[j] == ("op", "="), toks[i:j + 1]
            e, j = expr_tokens(toks, j + 1)
            qual = "const auto" if v == "let" else "auto"
            if ctype:
                out.append(f"{ctype} {name} = {emit_expr(e)};")
            else:
                out.append(f"{qual} {name} = value({emit_expr(e)});")
            i = j + 1
        elif v == "for" and k == "id":
            # for (var n = e; cond; step) { ... }
            assert toks[i + 1] == ("op", "(") and toks[i + 2] == ("id", "var")
            name = toks[i + 3][1]
            assert toks[i + 4] == ("op", "=")
            init, j = expr_tokens(toks, i + 5)
            cond, j = expr_tokens(toks, j + 1)
            step, j = expr_tokens(toks, j + 1, stop=(")",))
            body, j = translate_body(toks, j + 1)
            out.append(f"for (auto {name} = {emit_expr(init)}; {emit_expr(cond)}; {emit_expr(step)}) {body}")
            i = j
        elif v == "if" and k == "id":
            cond, j = expr_tokens(toks, i + 1, stop=("{",))
            body, j = translate_body(toks, j)
            out.append(f"if ({emit_expr(cond)}) {body}")
            i = j
            while toks[i] == ("id", "else"):
                if toks[i + 1] == ("id", "if"):
                    cond, j = expr_tokens(toks, i + 2, stop=("{",))
                    body, j = translate_body(toks, j)
                    out.append(f"else if ({emit_expr(cond)}) {body}")
                else:
                    body, j = translate_body(toks, i + 1)
                    out.append(f"else {body}")
                i = j
        elif v == "return" and k == "id":
            e, j = expr_tokens(toks, i + 1)
            out.append(f"return {emit_expr(e)};" if e else "return;")
            i = j + 1
        else:
            e, j = expr_tokens(toks, i)
            out.append(emit_expr(e) + ";")
            i = j + 1
    return "\n".join(out) + "\n}", i + 1


def translate(src):
    """Module-scope declarations in C++ order (WGSL allows any order):
    structs, constants and resources, function prototypes, function bodies."""
    toks = fold_constants(tokenize(src))
    structs, decls, protos, funcs = [], [], [], []
    i = 0
    while i < len(toks):
        i = skip_attrs(toks, i)
        if i >= len(toks):
            break
        k, v = toks[i]
        if v == "const":
            name = toks[i + 1][1]
            assert toks[i + 2] == ("op", ":")
            t, j = parse_type(toks, i + 3)
            assert toks[j] == ("op", "=")
            e, j = expr_tokens(toks, j + 1)
            decls.append(f"static const {t} {name} = {emit_expr(e)};")
            i = j + 1
        elif v == "struct":
            name = toks[i + 1][1]
            assert toks[i + 2] == ("op", "{")
            j = i + 3
            fields = []
            while toks[j] != ("op", "}"):
                fname = toks[j][1]
                assert toks[j + 1] == ("op", ":")
                t, j = parse_type(toks, j + 2)
                fields.append(f"    {t} {fname};")
                if toks[j] == ("op", ","):
                    j += 1
            j += 1
            if j < len(toks) and toks[j] == ("op", ";"):
                j += 1
            structs.append(f"struct {name} {{\n" + "\n".join(fields) + "\n};")
            i = j
        elif v == "var":
            # var<storage, read_write> NAME: array<T>;  |  var<uniform> NAME: T;  |  var NAME: T;
            j = i + 1
            if toks[j] == ("op", "<"):
                while toks[j] != ("op", ">"):
                    j += 1
                j += 1
            name = toks[j][1]
            assert toks[j + 1] == ("op", ":")
            t, j = parse_type(toks, j + 2)
            assert toks[j] == ("op", ";")
            decls.append(f"static {t} {name};")
            i = j + 1
        elif v == "fn":
            name = toks[i + 1][1]
            cname = "wgsl_main" if name == "main" else name
            assert toks[i + 2] == ("op", "(")
            j = i + 3
            params = []
            while toks[j] != ("op", ")"):
                j = skip_attrs(toks, j)
                pname = toks[j][1]
                assert toks[j + 1] == ("op", ":")
                t, j = parse_type(toks, j + 2)
                params.append(f"{t} {pname}")
                if toks[j] == ("op", ","):
                    j += 1
            j += 1
            ret = "void"
            if toks[j] == ("op", "->"):
                ret, j = parse_type(toks, j + 1)
            body, j = translate_body(toks, j)
            protos.append(f"static {ret} {cname}({', '.join(params)});")
            funcs.append(f"static {ret} {cname}({', '.join(params)}) {body}")
            i = j
        else:
            raise SyntaxError(f"unsupported top-level token {toks[i]}")
    return "\n\n".join(structs + decls + ["\n".join(protos)] + funcs) + "\n"


HEADER = """// Generated by oracle/wgsl/translate.py from the reference's src/{name}.
// Not part of the repository: rebuilt from the reference's source by
// oracle/build_oracle.py.  Include inside a namespace that uses wgsl::.
"""

if __name__ == "__main__":
    src_path, out_path = sys.argv[1], sys.argv[2]
    with open(src_path) as f:
        code = translate(f.read())
    with open(out_path, "w") as f:
        f.write(HEADER.format(name=src_path.replace("\\", "/").rsplit("/", 1)[-1]) + code)
