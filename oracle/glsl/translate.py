"""Rewrite a GLSL compute shader into C++ against oracle/glsl/glsl.hpp.

Test infrastructure only.  The rewrite is mechanical and covers the subset
of GLSL the reference's compute shaders use: `#include` is inlined,
`#version`/`#pragma`/`#extension` and the workgroup-size declaration are
dropped, uniform blocks become global structs (a block without an instance
name becomes its members), opaque uniforms become globals the caller sets,
specialisation constants take the pipeline's values, `in`/`out`/`inout` parameters become values
or references, multi-component swizzles become member calls (`v.xyz` ->
`v.xyz()`, and the compound assignment `v.xyz op= e` -> `v.set_xyz(v.xyz()
op (e))`), `shared` variables become globals, constant arrays become `carray`s (an
index past the end reads a zero element instead of memory outside the
array), vector constructors whose arguments draw random numbers use braces
(C++ then evaluates them left to right, as GLSL does), and `main` is renamed
`shader_main`.  Nothing else of the source changes.
"""
from __future__ import annotations

import re
from pathlib import Path

_INCLUDE = re.compile(r'^\s*#\s*include\s+"([^"]+)"\s*$', re.M)
_DROP_LINE = re.compile(r'^\s*#\s*(version|pragma|extension)\b.*$', re.M)
_LOCAL_SIZE = re.compile(r'layout\s*\(\s*local_size[^)]*\)\s*in\s*;')
_BLOCK = re.compile(r'layout\s*\([^)]*\)\s*uniform\s+(\w+)\s*\{(.*?)\}\s*(\w*)\s*;', re.S)
_OPAQUE = re.compile(r'layout\s*\([^)]*\)\s*((?:restrict|writeonly|readonly|coherent)\s+)*uniform\s+(\w+)\s+(\w+)\s*;')
_SPEC_CONST = re.compile(r'layout\s*\(\s*constant_id\s*=\s*\d+\s*\)\s*const\s+(\w+)\s+(\w+)\s*=\s*([^;]+);')
_OUT_PARAM = re.compile(r'\b(?:inout|out)\s+(\w+)\s+(\w+)\b')
_IN_PARAM = re.compile(r'(?<=[(,])\s*in\s+(\w+)\s+(\w+)\b')
_SWZ_ASSIGN = re.compile(r'([A-Za-z_][\w.\[\]]*)\.(xyz|rgb)\s*([-+*/])=\s*([^;]+);')
_SWZ = re.compile(r'\.(xyzw|rgba|xyz|rgb|xy|rg)\b(?!\s*\()')
_SHARED = re.compile(r'^\s*shared\s+', re.M)
_MAIN = re.compile(r'\bvoid\s+main\s*\(\s*\)')
_QUALIFIERS = re.compile(r'\b(highp|mediump|lowp|precise)\s+')
_CONST_ARRAY = re.compile(r'\bconst\s+(\w+)\s+(\w+)\s*\[\s*(\w+)\s*\]\s*=')
_CTOR = re.compile(r'\b[iub]?vec[234]\(')
_DRAWS = re.compile(r'\b(pcg|randomFloat|rotatedRandom)\s*\(')


def braced_draws(src: str) -> str:
    """GLSL evaluates call arguments left to right; C++ leaves the order of
    a call's arguments unspecified but evaluates a braced list left to right.
    A vector constructor whose arguments draw random numbers (each draw
    advances the generator's state) is therefore written with braces."""
    out, i = [], 0
    for m in _CTOR.finditer(src):
        if m.start() < i:
            continue
        depth, j = 1, m.end()
        while depth and j < len(src):
            depth += {"(": 1, ")": -1}.get(src[j], 0)
            j += 1
        args = src[m.end():j - 1]
        if len(_DRAWS.findall(args)) > 1:
            out.append(src[i:m.end() - 1] + "{" + args + "}")
            i = j
    out.append(src[i:])
    return "".join(out)


def inline_includes(path: Path, seen: tuple = ()) -> str:
    text = path.read_text()

    def sub(m):
        inc = (path.parent / m.group(1)).resolve()
        if inc in seen:
            return ""
        return inline_includes(inc, seen + (inc,))

    return _INCLUDE.sub(sub, text)


def translate(path: Path, spec: dict | None = None) -> str:
    """spec: values of specialisation constants by name (the pipeline's
    VkSpecializationInfo); the others keep their default."""
    src = inline_includes(Path(path).resolve())
    src = _DROP_LINE.sub("", src)
    src = _LOCAL_SIZE.sub("", src)

    def block(m):
        name, body, inst = m.group(1), m.group(2), m.group(3)
        return f"struct {name} {{{body}}} {inst};" if inst else body

    src = _BLOCK.sub(block, src)
    src = _OPAQUE.sub(lambda m: f"{m.group(2)} {m.group(3)};", src)
    spec = spec or {}
    src = _SPEC_CONST.sub(lambda m: f"const {m.group(1)} {m.group(2)} = {spec.get(m.group(2), m.group(3))};", src)
    src = _OUT_PARAM.sub(lambda m: f"{m.group(1)}& {m.group(2)}", src)
    src = _IN_PARAM.sub(lambda m: f" {m.group(1)} {m.group(2)}", src)
    src = _SWZ_ASSIGN.sub(lambda m: f"{m.group(1)}.set_{m.group(2)}({m.group(1)}.{m.group(2)}() {m.group(3)} ({m.group(4)}));",
                          src)
    src = _SWZ.sub(lambda m: f".{m.group(1)}()", src)
    src = _SHARED.sub("", src)
    src = _MAIN.sub("void shader_main()", src)
    src = _QUALIFIERS.sub("", src)
    src = _CONST_ARRAY.sub(lambda m: f"const carray<{m.group(1)}, {m.group(3)}> {m.group(2)} =", src)
    src = braced_draws(src)
    return src


if __name__ == "__main__":
    import sys
    print(translate(Path(sys.argv[1])))
