"""Translates the reference's Slang compute shaders, token by token, into C++
that compiles against oracle/slang_cpu.h, so that the shaders' own source
runs on the CPU.

TEST INFRASTRUCTURE ONLY: run by oracle/build_ref.py where the reference tree
is present; the generated files go to oracle/_ref/gen/ (git-ignored) and build
the checker library oracle/_ref/libtpdref.so. Nothing here is product code.

The translation is mechanical; each rule maps one Slang construct to the C++
construct with the same meaning (slang_cpu.h gives the types, intrinsics and
the workgroup execution model):

  import splat; / module / implementing  the module's text, translated, included once per shader
  __include "f"                          the translated text of f, inline
  public, uniform, attributes ([[...]], [shader], [numthreads], [SpecializationConstant])
                                         dropped ([numthreads] is kept as the shader's workgroup size)
  groupshared                            thread_local (a workgroup runs on one host thread)
  let x = e / var x = e                  const auto x = e / auto x = e
  out T x / inout T x (parameters)       T& x
  v.xy / v.xyz (swizzles)                v.xy() / v.xyz()
  1.5 (a float literal)                  1.5f  (Slang literals are 32-bit floats)
  T::maxValue                            std::numeric_limits<T>::max()
  (int)(e)                               to_int(e)  (saturating truncation)
  a trailing comma before )              removed
  struct S { ... }                       struct S { ... };
  ConstantBuffer<float4[4]>.Handle       TransformHandle (bindless model matrix)
  void main(T a : SV_X, ...)             void shader_main(T a, ...) plus entry(gtid, gid, dtid)
                                         passing each parameter by its semantic

Each generated file starts with #line directives, so compiler messages point
at the Slang source lines.
"""
from __future__ import annotations

import re
from pathlib import Path

SEMANTICS = {"SV_GroupThreadID": "gtid", "SV_GroupID": "gid", "SV_DispatchThreadID": "dtid"}


def _float_literals(text: str) -> str:
    # a decimal literal with a point and no suffix is a 32-bit float in Slang
    return re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][-+]?\d+)?(?![\w.])", lambda m: m.group(0) + "f", text)


def _translate_code(code: str) -> str:
    code = re.sub(r"\bConstantBuffer<float4\[4\]>\.Handle\b", "TransformHandle", code)
    code = re.sub(r"\b(public|uniform)\s+", "", code)
    code = re.sub(r"\bgroupshared\s+", "thread_local ", code)
    code = re.sub(r"\blet\s+", "const auto ", code)
    code = re.sub(r"\bvar\s+", "auto ", code)
    code = re.sub(r"([(,])([ \t]*)(?:out|inout)[ \t]+(\w+)[ \t]+(\w+)", r"\1\2\3& \4", code)
    code = re.sub(r"\.(xyz|xy)\b(?!\s*\()", r".\1()", code)
    code = re.sub(r"\b(\w+)::maxValue\b", r"std::numeric_limits<\1>::max()", code)
    code = re.sub(r"\(int\)\(", "to_int(", code)
    return _float_literals(code)


def _close_structs(text: str) -> str:
    out, i = [], 0
    for m in re.finditer(r"\bstruct\s+\w+\s*\{", text):
        if m.start() < i:
            continue
        depth, j = 0, m.end() - 1
        while j < len(text):
            if text[j] == "{":
                depth += 1
            elif text[j] == "}":
                depth -= 1
                if depth == 0:
                    break
            j += 1
        out.append(text[i:j + 1])
        rest = text[j + 1:]
        if not rest.lstrip().startswith(";"):
            out.append(";")
        i = j + 1
    out.append(text[i:])
    return "".join(out)


def translate_text(text: str) -> tuple[str, tuple[str, ...] | None, list[tuple[str, str]] | None]:
    """Slang text -> (C++ text, numthreads expressions or None, main's (param, semantic) list or None)."""
    numthreads = None
    m = re.search(r"\[numthreads\(([^)]*)\)\]", text)
    if m:
        numthreads = tuple(x.strip() for x in m.group(1).split(","))
    lines = []
    for line in text.splitlines():
        s = line.strip()
        if re.match(r"^(module|implementing)\s+\w+\s*;", s) or re.match(r"^import\s+\w+\s*;", s):
            lines.append("// " + s)
            continue
        # attributes on their own line
        line = re.sub(r"\[\[[^\]]*\]\]", "", line)
        line = re.sub(r"^\s*\[(shader|numthreads|SpecializationConstant)[^\]]*\]\s*$", "", line)
        line = re.sub(r"^\s*\[(shader|numthreads|SpecializationConstant)[^\]]*\]", "", line)
        lines.append(line)
    text = "\n".join(lines)
    # token rules apply to code only; comments are kept as they are
    parts = re.split(r"(//[^\n]*|/\*.*?\*/)", text, flags=re.S)
    for k in range(0, len(parts), 2):
        parts[k] = _translate_code(parts[k])
    text = "".join(parts)
    text = re.sub(r",(\s*)\)", r"\1)", text)  # a trailing argument comma may precede a comment
    text = _close_structs(text)
    params = None
    m = re.search(r"\bvoid\s+main\s*\(([^)]*)\)", text)
    if m:
        params = []
        plist = []
        for p in m.group(1).split(","):
            pm = re.match(r"\s*(\w+)\s+(\w+)\s*:\s*(\w+)\s*$", p)
            if not pm:
                raise ValueError(f"unhandled main parameter: {p!r}")
            params.append((pm.group(2), pm.group(3)))
            plist.append(f"{pm.group(1)} {pm.group(2)}")
        text = text[:m.start()] + "void shader_main(" + ", ".join(plist) + ")" + text[m.end():]
    return text, numthreads, params


_FUNC_DEF = re.compile(r"^([A-Za-z_][\w<>]*)\s+([A-Za-z_]\w*)\s*\(([^;{()]*(?:\[\])?[^;{()]*)\)\s*\{", re.M)


def _prototypes(text: str) -> str:
    """Declarations of the functions a text defines (Slang declarations are
    order-free; C++ needs a function declared before its first call)."""
    protos = []
    for m in _FUNC_DEF.finditer(text):
        if m.group(1) in ("struct", "return", "else", "if", "for", "while", "switch"):
            continue
        protos.append(f"{m.group(1)} {m.group(2)}({m.group(3)});")
    return "\n".join(protos)


def translate_module(root: Path) -> str:
    """splat.slang with its __include'd files, as one C++ text: the module's
    own constants and structs first, then the declarations of every function,
    then the included files' bodies (Slang modules are order-free)."""
    main = root / "splat.slang"
    text = main.read_text()
    incs = [root / f for f in re.findall(r'^\s*__include\s+"([^"]+)"\s*;', text, re.M)]
    own = re.sub(r'^\s*__include\s+"[^"]+"\s*;', lambda m: "// " + m.group(0).strip(), text, flags=re.M)
    own_cpp, _, _ = translate_text(own)
    bodies = [(inc, translate_text(inc.read_text())[0]) for inc in incs]
    out = [f'#line 1 "{main}"', own_cpp, "#line 1 \"<declarations>\""]
    out += [_prototypes(b) for _, b in bodies]
    for inc, b in bodies:
        out += [f'#line 1 "{inc}"', b]
    return "\n".join(out) + "\n"


def translate_shader(path: Path) -> str:
    """One compute shader as C++: its translated text, its workgroup size and
    an entry(gtid, gid, dtid) that calls shader_main with its semantics."""
    body, numthreads, params = translate_text(path.read_text())
    if numthreads is None or params is None:
        raise ValueError(f"{path}: no [numthreads] or no main")
    defines = re.findall(r"^\s*#define\s+(\w+)", body, re.M)
    args = ", ".join(SEMANTICS[sem] for _, sem in params)
    tail = [
        f"inline uint3 numthreads() {{ return uint3(uint({numthreads[0]}), uint({numthreads[1]}), "
        f"uint({numthreads[2]})); }}",
        f"inline void entry(uint3 gtid, uint3 gid, uint3 dtid) {{ (void)gtid; (void)gid; (void)dtid; "
        f"shader_main({args}); }}",
    ]
    tail += [f"#undef {d}" for d in defines]
    return f'#include "splat_module.inc"\n#line 1 "{path}"\n' + body + "\n" + "\n".join(tail) + "\n"


SHADERS = ("project", "prefix", "keygen", "radix-shuffle", "radix-prefixA", "radix-prefixB", "radix-mapping",
           "range", "blend")


def generate(shader_root: Path, out_dir: Path) -> list[Path]:
    """Writes splat_module.inc and one <shader>.inc per shader into out_dir."""
    out_dir.mkdir(parents=True, exist_ok=True)
    written = []
    mod = out_dir / "splat_module.inc"
    mod.write_text("// generated by oracle/slang_to_cpp.py from the reference's splat module\n" +
                   translate_module(shader_root))
    written.append(mod)
    for name in SHADERS:
        f = out_dir / f"{name.replace('-', '_')}.inc"
        f.write_text(f"// generated by oracle/slang_to_cpp.py from {name}.slang\n" +
                     translate_shader(shader_root / f"{name}.slang"))
        written.append(f)
    return written
