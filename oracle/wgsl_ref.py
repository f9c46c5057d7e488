"""The reference's own simulation kernels on the CPU — TEST INFRASTRUCTURE ONLY.

The reference's substep is WGSL (web/js/shaders/common.js:11-397 and
web/js/shaders/simkernels.js:15-544, embedded in JavaScript template
strings). No WebGPU adapter exists on either machine, so this script
translates that WGSL mechanically into C++ — the same functions, statements
and expressions, token by token, with no hand edits — and compiles it with
oracle/wgsl_rt.h (WGSL types, abstract-float evaluation, builtins, atomics
in invocation order, workgroup barriers as coroutine suspensions) and oracle/wgsl_ref.cpp
(the dispatch sequence of web/js/sim.js:220-272) into oracle/_ref/.

Outputs, all under oracle/_ref/ (git-ignored; the generated source travels
with the working tree so the library can be rebuilt on another host):
    xpbi_wgsl.inc      the translated shader module
    libxpbi_wgslref.so the reference kernels behind wr_substep()

translate() needs the reference checkout: the directory XPBI_REFERENCE
names, else a checkout named `reference` beside this repository; build()
needs only the generated source.
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
INC = os.path.join(OUT, "xpbi_wgsl.inc")
LIB = os.path.join(OUT, "libxpbi_wgslref.so")
DRIVER = os.path.join(HERE, "wgsl_ref.cpp")
RUNTIME = os.path.join(HERE, "wgsl_rt.h")
SHADERS = ("web/js/shaders/common.js", "web/js/shaders/simkernels.js")


def reference_root() -> str:
    """The reference checkout: XPBI_REFERENCE, else `reference` beside this
    repository's root."""
    env = os.environ.get("XPBI_REFERENCE")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


# ------------------------------------------------------------------ extraction
def extract_wgsl(js: str) -> str:
    """The bodies of the /* wgsl */ template literals of one module."""
    out = []
    for m in re.finditer(r"/\*\s*wgsl\s*\*/\s*`", js):
        end = js.index("`", m.end())
        body = js[m.end():end]
        if "${" in body:
            raise ValueError("template interpolation in WGSL source")
        out.append(body)
    if not out:
        raise ValueError("no WGSL template found")
    return "\n".join(out)


# ------------------------------------------------------------------ tokens
_TOKEN = re.compile(r"""
  (?P<nl>\n) | (?P<ws>[ \t\r]+) | (?P<com>//[^\n]*) | (?P<bcom>/\*.*?\*/) |
  (?P<num>0[xX][0-9a-fA-F]+[iu]? | (?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?[fh]? | \d+[eE][+-]?\d+[fh]? | \d+[iuf]?) |
  (?P<id>[A-Za-z_]\w*) |
  (?P<op>->|<<=|>>=|<<|>>|<=|>=|==|!=|&&|\|\||\+\+|--|[-+*/%&|^]=|[-+*/%<>=!&|^~?:;,.(){}\[\]@])
""", re.X | re.S)


class Tok:
    __slots__ = ("kind", "text")

    def __init__(self, kind, text):
        self.kind, self.text = kind, text

    def __repr__(self):
        return f"{self.kind}:{self.text}"


def tokenize(src: str) -> list[Tok]:
    toks, pos = [], 0
    while pos < len(src):
        m = _TOKEN.match(src, pos)
        if not m:
            raise ValueError(f"cannot tokenize at {src[pos:pos + 40]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind in ("ws", "com", "bcom", "nl"):
            continue
        toks.append(Tok(kind, m.group()))
    return toks


# identifiers of the WGSL module that would collide with C++ or the runtime
_RENAME = {
    "auto", "char", "class", "delete", "double", "enum", "explicit", "export", "extern", "float", "friend",
    "goto", "inline", "int", "long", "mutable", "namespace", "new", "operator", "private", "protected",
    "public", "register", "short", "signed", "sizeof", "static", "template", "this", "throw", "try", "catch",
    "typedef", "typeid", "typename", "union", "unsigned", "using", "virtual", "void", "volatile", "and", "or",
    "not", "xor", "compl", "bitand", "bitor", "AF", "V2", "V3", "V4", "WArr", "concretize", "vmap", "vzip",
    "unify", "elem", "is_vec", "min_impl", "max_impl", "pow_impl", "loadField", "runWorkgroup", "EntryFn",
    "FiberPool", "fiberPool", "fiberEntry", "wgsl", "std",
}
_UNSUPPORTED = {"loop", "continuing", "discard", "fallthrough", "bitcast", "override", "diagnostic"}
_SWIZZLE = re.compile(r"[xyzw]{2,4}$")
_RMW = {"atomicAdd", "atomicSub", "atomicMax", "atomicMin", "atomicAnd", "atomicOr", "atomicXor",
        "atomicExchange", "atomicCompareExchangeWeak"}
_BUILTIN_PARAMS = {"global_invocation_id": 0, "local_invocation_id": 1, "workgroup_id": 2}


def num(t: str) -> str:
    """A WGSL literal as C++: abstract floats become AF(...), f32 literals
    keep f, u32 keep u, i32 and abstract ints are plain ints."""
    if t.lower().startswith("0x"):
        return t[:-1] if t.endswith("i") else t
    if t.endswith("h"):
        raise ValueError("f16 literal")
    is_float = ("." in t) or ("e" in t.lower()) or t.endswith("f")
    if is_float:
        if t.endswith("f"):
            body = t[:-1]
            return body + ("f" if ("." in body or "e" in body.lower()) else ".0f")
        return f"AF({t})"
    if t.endswith("u"):
        return t
    if t.endswith("i"):
        return t[:-1]
    return t


def ident(t: str) -> str:
    if t in _UNSUPPORTED:
        raise ValueError(f"unsupported WGSL construct: {t}")
    return t + "_w" if t in _RENAME else t


class Translator:
    def __init__(self, toks: list[Tok]):
        self.t = toks
        self.consts: list[str] = []
        self.structs: list[str] = []
        self.struct_fields: dict[str, list[tuple[str, list[Tok]]]] = {}
        self.globals: list[str] = []
        self.protos: list[str] = []
        self.funcs: list[str] = []
        self.entries: list[tuple[str, str, bool, bool]] = []   # name, wg expr, barrier, rmw atomics
        self.uniforms: list[tuple[str, list[Tok]]] = []
        self.storage: list[tuple[str, str]] = []               # name, element C++ type
        self.workgroup: list[str] = []

    # -------------------------------------------------------------- helpers
    def expect(self, i, text):
        if self.t[i].text != text:
            ctx = " ".join(x.text for x in self.t[max(0, i - 8):i + 8])
            raise ValueError(f"expected {text!r} at token {i}: ... {ctx} ...")
        return i + 1

    def match(self, i, open_, close):
        depth = 0
        for k in range(i, len(self.t)):
            if self.t[k].text == open_:
                depth += 1
            elif self.t[k].text == close:
                depth -= 1
                if depth == 0:
                    return k
        raise ValueError(f"unbalanced {open_}")

    def attrs(self, i):
        out = []
        while i < len(self.t) and self.t[i].text == "@":
            name = self.t[i + 1].text
            i += 2
            args = []
            if i < len(self.t) and self.t[i].text == "(":
                j = self.match(i, "(", ")")
                args = self.t[i + 1:j]
                i = j + 1
            out.append((name, args))
        return out, i

    def parse_type(self, i):
        """Returns (C++ type, kind, element C++ type, WGSL tokens, next index).
        kind is 'rtarray' for a runtime-sized array (a storage pointer)."""
        start = i
        name = self.t[i].text
        i += 1
        if i < len(self.t) and self.t[i].text == "<":
            # template arguments; '>>' closes two levels
            depth, args, cur, k = 1, [], [], i + 1
            while depth:
                tx = self.t[k].text
                if tx == "<":
                    depth += 1
                    cur.append(self.t[k])
                elif tx in (">", ">>"):
                    closes = 1 if tx == ">" else 2
                    for _ in range(closes):
                        depth -= 1
                        if depth == 0:
                            break
                        cur.append(Tok("op", ">"))
                    if depth == 0:
                        args.append(cur)
                        break
                elif tx == "," and depth == 1:
                    args.append(cur)
                    cur = []
                else:
                    cur.append(self.t[k])
                k += 1
            i = k + 1
            wgsl_toks = self.t[start:i]
            if name == "array":
                et, _, _, _, _ = Translator(args[0] + [Tok("op", ";")]).parse_type(0)
                if len(args) == 1:
                    return et + "*", "rtarray", et, wgsl_toks, i
                n = " ".join(num(x.text) if x.kind == "num" else ident(x.text) for x in args[1])
                return f"WArr<{et}, {n}>", "array", et, wgsl_toks, i
            if name == "atomic":
                et, _, _, _, _ = Translator(args[0] + [Tok("op", ";")]).parse_type(0)
                return et, "scalar", et, wgsl_toks, i
            if name == "ptr":
                et, _, _, _, _ = Translator(args[1] + [Tok("op", ";")]).parse_type(0)
                return et + "*", "ptr", et, wgsl_toks, i
            if name in ("vec2", "vec3", "vec4"):
                et, _, _, _, _ = Translator(args[0] + [Tok("op", ";")]).parse_type(0)
                return f"V{name[3]}<{et}>", "vec", et, wgsl_toks, i
            raise ValueError(f"unsupported template type {name}")
        return ident(name), "plain", ident(name), self.t[start:i], i

    # -------------------------------------------------------------- expressions / bodies
    def stmt_end(self, i):
        depth = 0
        for k in range(i, len(self.t)):
            tx = self.t[k].text
            if tx in "([{":
                depth += 1
            elif tx in ")]}":
                depth -= 1
            elif tx == ";" and depth == 0:
                return k
        raise ValueError("statement without ';'")

    def expr(self, a, b) -> str:
        return self.body(a, b)

    def body(self, a, b) -> str:
        """Statements / expressions of tokens [a, b) as C++."""
        out, i = [], a
        while i < b:
            tk = self.t[i]
            tx = tk.text
            if tk.kind == "num":
                out.append(num(tx))
                i += 1
                continue
            if tx in ("let", "var") and tk.kind == "id":
                is_let = tx == "let"
                i += 1
                if self.t[i].text == "<":
                    raise ValueError("address-space var inside a function")
                name = ident(self.t[i].text)
                i += 1
                ctype = None
                if self.t[i].text == ":":
                    ctype, _, _, _, i = self.parse_type(i + 1)
                end = self.stmt_end(i)
                if self.t[i].text == "=":
                    init = self.expr(i + 1, end)
                    if ctype:
                        out.append(f"{'const ' if is_let else ''}{ctype} {name} = {init};")
                    else:
                        out.append(f"{'const ' if is_let else ''}auto {name} = concretize({init});")
                else:
                    if is_let or not ctype:
                        raise ValueError("declaration without initializer or type")
                    out.append(f"{ctype} {name}{{}};")
                i = end + 1
                continue
            if tx in ("case", "default") and tk.kind == "id":
                # case selectors: WGSL lists them with commas, the ':' is optional
                k = i + 1
                sels, cur = [], []
                while self.t[k].text not in ("{", ":"):
                    if self.t[k].text == ",":
                        sels.append(cur)
                        cur = []
                    else:
                        cur.append(self.t[k])
                    k += 1
                if cur:
                    sels.append(cur)
                if self.t[k].text == ":":
                    k += 1
                if tx == "default":
                    labels = "default:"
                else:
                    labels = " ".join("case " + " ".join(num(x.text) if x.kind == "num" else ident(x.text)
                                                          for x in s) + ":" for s in sels)
                if self.t[k].text != "{":
                    raise ValueError("case without a block")
                j = self.match(k, "{", "}")
                out.append(labels + " {" + self.body(k + 1, j) + "} break;")
                i = j + 1
                continue
            if tx == "." and i + 1 < b and self.t[i + 1].kind == "id" and _SWIZZLE.match(self.t[i + 1].text):
                sw = self.t[i + 1].text
                if sw != "xyz":
                    raise ValueError(f"unsupported swizzle .{sw}")
                out.append(".xyz()")
                i += 2
                continue
            if tx == "@":
                raise ValueError("attribute inside a function body")
            out.append(ident(tx) if tk.kind == "id" else tx)
            i += 1
            if tx in ("{", "}", ";"):
                out.append("\n")
        return " ".join(out).replace(" \n ", "\n").replace("\n ", "\n")

    # -------------------------------------------------------------- declarations
    def run(self):
        i = 0
        pending = []
        while i < len(self.t):
            tx = self.t[i].text
            if tx == "@":
                a, i = self.attrs(i)
                pending += a
                continue
            if tx == ";":
                i += 1
                continue
            if tx == "struct":
                i = self.struct(i)
            elif tx == "const":
                i = self.const(i)
            elif tx == "var":
                i = self.global_var(i, pending)
            elif tx == "fn":
                i = self.function(i, pending)
            else:
                raise ValueError(f"unexpected top-level token {tx!r}")
            pending = []
        return self

    def struct(self, i):
        name = ident(self.t[i + 1].text)
        i = self.expect(i + 2, "{")
        j = self.match(i - 1, "{", "}")
        fields = []
        k = i
        while k < j:
            _, k = self.attrs(k)
            if k >= j:
                break
            fname = ident(self.t[k].text)
            k = self.expect(k + 1, ":")
            ctype, _, _, wt, k = self.parse_type(k)
            fields.append((fname, ctype, wt))
            if self.t[k].text == ",":
                k += 1
        self.struct_fields[name] = [(f, wt) for f, _, wt in fields]
        decl = [f"struct {name} {{"]
        decl += [f"  {ct} {fn}{{}};" for fn, ct, _ in fields]
        decl.append(f"  {name}() = default;")
        params = ", ".join(f"const {ct}& {fn}_" for fn, ct, _ in fields)
        inits = ", ".join(f"{fn}({fn}_)" for fn, _, _ in fields)
        decl.append(f"  {name}({params}) : {inits} {{}}")
        decl.append("};")
        self.structs.append("\n".join(decl))
        i = j + 1
        if i < len(self.t) and self.t[i].text == ";":
            i += 1
        return i

    def const(self, i):
        name = ident(self.t[i + 1].text)
        i += 2
        ctype = None
        if self.t[i].text == ":":
            ctype, _, _, _, i = self.parse_type(i + 1)
        i = self.expect(i, "=")
        end = self.stmt_end(i)
        init = self.expr(i, end)
        self.consts.append(f"static const {ctype or 'auto'} {name} = {init};")
        return end + 1

    def global_var(self, i, attrs):
        i += 1
        space = []
        if self.t[i].text == "<":
            j = self.match(i, "<", ">")
            space = [x.text for x in self.t[i + 1:j] if x.text != ","]
            i = j + 1
        name = ident(self.t[i].text)
        i = self.expect(i + 1, ":")
        ctype, kind, etype, wt, i = self.parse_type(i)
        if self.t[i].text == "=":
            raise ValueError("initialised module-scope var")
        i = self.expect(i, ";")
        sp = space[0] if space else "private"
        if sp == "uniform":
            self.globals.append(f"static {ctype} {name};")
            self.uniforms.append((name, wt))
        elif sp == "storage":
            if kind != "rtarray":
                raise ValueError("storage binding that is not a runtime-sized array")
            self.globals.append(f"static {ctype} {name} = nullptr;")
            self.storage.append((name, etype))
        elif sp == "workgroup":
            self.globals.append(f"static thread_local {ctype} {name};")
            self.workgroup.append(name)
        else:
            self.globals.append(f"static thread_local {ctype} {name}{{}};")
        return i

    def function(self, i, attrs):
        name = ident(self.t[i + 1].text)
        i = self.expect(i + 2, "(")
        j = self.match(i - 1, "(", ")")
        params = []
        builtins = {}
        k = i
        while k < j:
            pa, k = self.attrs(k)
            pname = ident(self.t[k].text)
            k = self.expect(k + 1, ":")
            ctype, _, _, _, k = self.parse_type(k)
            bi = [a for a in pa if a[0] == "builtin"]
            if bi:
                which = bi[0][1][0].text
                if which not in _BUILTIN_PARAMS:
                    raise ValueError(f"unsupported builtin {which}")
                builtins[_BUILTIN_PARAMS[which]] = pname
            else:
                params.append(f"{ctype} {pname}")
            if self.t[k].text == ",":
                k += 1
        i = j + 1
        ret = "void"
        if self.t[i].text == "->":
            _, i = self.attrs(i + 1)
            ret, _, _, _, i = self.parse_type(i)
        b0 = self.expect(i, "{")
        b1 = self.match(i, "{", "}")
        body_toks = self.t[b0:b1]
        text = self.body(b0, b1)
        entry = any(a[0] == "compute" for a in attrs)
        barrier = any(x.text == "workgroupBarrier" for x in body_toks)
        if barrier:
            if not entry:
                raise ValueError("workgroupBarrier outside an entry point")
            # a coroutine: each barrier suspends the invocation
            text = re.sub(r"\bworkgroupBarrier \( \) ;", "co_await Barrier{} ;", text)
            text = re.sub(r"\breturn ;", "co_return ;", text)
        if entry:
            names = [builtins.get(k, f"unused{k}_") for k in range(3)]
            rtype = "WgTask" if barrier else "void"
            sig = f"static {rtype} {name}(vec3u {names[0]}, vec3u {names[1]}, vec3u {names[2]})"
            wg = [a for a in attrs if a[0] == "workgroup_size"]
            if not wg:
                raise ValueError(f"entry point {name} without workgroup_size")
            wg_expr = " ".join(num(x.text) if x.kind == "num" else ident(x.text) for x in wg[0][1])
            if "," in wg_expr:
                raise ValueError("multi-dimensional workgroups")
            # read-modify-write atomics make the invocation order matter: such
            # kernels run their invocations one at a time, in index order
            rmw = any(x.text in _RMW for x in body_toks)
            self.entries.append((name, wg_expr, barrier, rmw))
        else:
            sig = f"static {ret} {name}({', '.join(params)})"
            self.protos.append(sig + ";")
        self.funcs.append(sig + " {\n" + text + "\n}")
        return b1 + 1

    # -------------------------------------------------------------- layout (WGSL uniform address space)
    def layout(self, wt: list[Tok]):
        """(align, size) of a WGSL type given by its tokens."""
        name = wt[0].text
        scal = {"f32": (4, 4), "u32": (4, 4), "i32": (4, 4)}
        if name in scal:
            return scal[name]
        if re.match(r"vec([234])[fiu]$", name):
            n = int(name[3])
            return {2: (8, 8), 3: (16, 12), 4: (16, 16)}[n]
        if name == "mat3x3f":
            return (16, 48)
        if name in self.struct_fields:
            off, al = 0, 1
            for _, fwt in self.struct_fields[name]:
                a, s = self.layout(fwt)
                off = (off + a - 1) // a * a + s
                al = max(al, a)
            return (al, (off + al - 1) // al * al)
        raise ValueError(f"no layout for {name}")

    def loader(self, sname: str) -> str:
        lines = [f"static void load_{sname}({sname}& s, const uint32_t* w) {{"]
        off = 0
        for fname, fwt in self.struct_fields[sname]:
            a, s = self.layout(fwt)
            off = (off + a - 1) // a * a
            if fwt[0].text in self.struct_fields:
                lines.append(f"  load_{fwt[0].text}(s.{fname}, w + {off // 4});")
            else:
                lines.append(f"  loadField(s.{fname}, w, {off});")
            off += s
        lines.append("}")
        return "\n".join(lines)

    def emit(self, origin: str) -> str:
        parts = [
            "// GENERATED by oracle/wgsl_ref.py from the reference's WGSL (" + origin + ").",
            "// Test infrastructure only; not product code. Do not edit: regenerate.",
            "namespace wgsl_ref {",
            "using namespace wgsl;",
        ]
        parts += self.consts + self.structs + self.globals + self.protos + self.funcs
        # uniform loaders
        for sname in self.struct_fields:
            try:
                self.layout([Tok("id", sname)])
            except ValueError:
                continue
            parts.append(self.loader(sname))
        lines = ["static void loadUniform(const char* name, const uint32_t* w) {"]
        for uname, wt in self.uniforms:
            if wt[0].text == "array":
                et = wt[2].text
                a, s = self.layout([Tok("id", et)])
                stride = (s + 15) // 16 * 16   # uniform arrays: element stride a multiple of 16
                n = wt[4].text
                lines.append(f'  if (!std::strcmp(name, "{uname}")) {{ for (int k = 0; k < {n}; ++k) '
                             f'load_{et}({uname}[k], w + k * {stride // 4}); return; }}')
            else:
                lines.append(f'  if (!std::strcmp(name, "{uname}")) {{ load_{wt[0].text}({uname}, w); return; }}')
        lines.append("}")
        parts.append("\n".join(lines))
        lines = ["static bool bindStorage(const char* name, void* p) {"]
        for sname, et in self.storage:
            lines.append(f'  if (!std::strcmp(name, "{sname}")) {{ {sname} = static_cast<{et}*>(p); return true; }}')
        lines.append("  return false;\n}")
        parts.append("\n".join(lines))
        parts.append("static void resetWorkgroupVars() {\n" +
                     "".join(f"  {w} = {{}};\n" for w in self.workgroup) + "}")
        parts.append("struct Entry { const char* name; EntryFn fn; BarrierFn co; u32 wg; bool serial; };")
        parts.append("static const Entry kEntries[] = {\n" + "".join(
            f'  {{"{n}", {"nullptr" if b else n}, {n if b else "nullptr"}, {wg}, {str(a).lower()}}},\n'
            for n, wg, b, a in self.entries) + "};")
        parts.append("}  // namespace wgsl_ref")
        return "\n\n".join(parts) + "\n"


def translate(ref: str | None = None) -> str:
    """Generates oracle/_ref/xpbi_wgsl.inc from the reference checkout."""
    ref = ref or reference_root()
    src = []
    for rel in SHADERS:
        with open(os.path.join(ref, rel)) as f:
            src.append(extract_wgsl(f.read()))
    tr = Translator(tokenize("\n".join(src))).run()
    os.makedirs(OUT, exist_ok=True)
    text = tr.emit(", ".join(SHADERS))
    tmp = INC + ".tmp"
    with open(tmp, "w") as f:
        f.write(text)
    os.replace(tmp, INC)
    return INC


def available() -> bool:
    return os.path.exists(INC) or os.path.isdir(os.path.join(reference_root(), "web/js/shaders"))


def build(force: bool = False) -> str | None:
    """Builds oracle/_ref/libxpbi_wgslref.so; returns its path, or None when
    neither the generated source nor the reference checkout is present."""
    if not os.path.exists(INC) or force:
        if not os.path.isdir(os.path.join(reference_root(), "web/js/shaders")):
            return None
        translate()
    deps = [INC, DRIVER, RUNTIME, __file__]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O3", "-std=c++20", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-shared", "-fPIC",
           "-I", HERE, "-I", OUT, DRIVER, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("WGSL reference build failed:\n" + " ".join(cmd) + "\n" + r.stdout[-4000:] +
                           r.stderr[-8000:])
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    """The reference kernels' library (built on first use)."""
    global _lib
    if _lib is None:
        path = build()
        if path is None:
            raise FileNotFoundError("the reference's WGSL is not available (no generated source, no checkout)")
        L = ctypes.CDLL(path)
        u32p, fp = ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_float)
        L.wr_substep.restype = ctypes.c_int
        L.wr_substep.argtypes = [u32p, u32p, ctypes.c_uint32, fp, fp, fp, fp, fp, u32p, u32p,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        _lib = L
    return _lib


def substep(params_words, material_words, state: dict, iterations: int, has_water: bool,
            pbf_iterations: int = -1, substeps: int = 1, threads: int = 0) -> dict:
    """`substeps` substeps of the reference's own kernels from `state` (the
    layouts of the oracle's substep()); returns the new state."""
    import numpy as np

    n = len(state["pos"])
    nc = int(params_words[7])
    out = {k: np.ascontiguousarray(state[k], np.float32).copy() for k in ("pos", "vel", "F", "aux")}
    out["L"] = (np.zeros((n, 12), np.float32) if state.get("L") is None
                else np.ascontiguousarray(state["L"], np.float32).copy())
    out["sortedIdx"] = np.zeros(n, np.uint32)
    out["cellTab"] = np.zeros(nc, np.uint32)
    pw = np.ascontiguousarray(params_words, np.uint32)
    mw = np.ascontiguousarray(material_words, np.uint32)

    def p(a, t):
        return a.ctypes.data_as(ctypes.POINTER(t))

    f, u = ctypes.c_float, ctypes.c_uint32
    rc = lib().wr_substep(p(pw, u), p(mw, u), n, p(out["pos"], f), p(out["vel"], f), p(out["F"], f),
                          p(out["L"], f), p(out["aux"], f), p(out["sortedIdx"], u), p(out["cellTab"], u),
                          iterations, 1 if has_water else 0, pbf_iterations, substeps, threads)
    if rc != 0:
        raise RuntimeError(f"reference substep failed ({rc})")
    return out


if __name__ == "__main__":
    if "--translate" in sys.argv:
        print(translate())
    print(build(force="--force" in sys.argv))
