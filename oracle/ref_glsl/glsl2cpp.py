"""Rewrite the reference's GLSL shader files into C++ includes.

TEST INFRASTRUCTURE ONLY (part of the oracle/_ref recipe).  Reads the
reference's shaders where they lie and writes oracle/_ref/glsl/<name>.inc.
The rewrite is mechanical; the shader code itself is left as written:
  * parameter qualifiers: ``inout T x`` / ``out T x`` -> ``T& x``, ``in T x`` -> ``T x``
  * ``uniform`` is dropped (uniforms become globals set by the driver)
  * the RNG state globals ``seed`` / ``pixel`` become thread_local
  * a call with two ``rand()`` arguments gets them evaluated left to right
    (GLSL's order; C++ leaves it unspecified)
  * tile.glsl: ``#version``, ``#include`` and the ``in``/``out`` interface
    lines are dropped and ``main`` becomes ``tile_main``
  * tonemap.glsl: likewise, and ``main`` becomes ``tonemap_main``
Usage: python glsl2cpp.py <shader_dir> <out_dir>
"""
import os
import re
import sys

FILES = [
    "common/uniforms.glsl",
    "common/globals.glsl",
    "common/intersection.glsl",
    "common/sampling.glsl",
    "common/envmap.glsl",
    "common/anyhit.glsl",
    "common/closest_hit.glsl",
    "common/disney.glsl",
    "common/lambert.glsl",
    "common/pathtrace.glsl",
    "tile.glsl",
    "tonemap.glsl",
]


def rewrite(text: str, name: str) -> str:
    out_lines = []
    for line in text.splitlines():
        s = line.strip()
        if name == "tile.glsl":
            if s.startswith("#version") or s.startswith("#include"):
                continue
            if s in ("out vec4 color;", "in vec2 TexCoords;"):
                continue
            line = line.replace("void main(void)", "void tile_main()")
        if name == "tonemap.glsl":
            if s.startswith("#version") or s.startswith("#include"):
                continue
            if s in ("out vec4 outCol;", "in vec2 TexCoords;"):
                continue
            line = line.replace("void main()", "void tonemap_main()")
        if s.startswith("uniform "):
            line = line.replace("uniform ", "", 1)
        if s == "uvec4 seed;":
            line = "thread_local uvec4 seed;"
        if s == "ivec2 pixel;":
            line = "thread_local ivec2 pixel;"
        # GLSL evaluates call arguments left to right; C++ leaves the order
        # unspecified, so calls taking two rand() arguments are sequenced.
        line = re.sub(r"(\w+)\(([^()]*), rand\(\), rand\(\)\)",
                      r"[&]{ float _ra = rand(); float _rb = rand(); return \1(\2, _ra, _rb); }()", line)
        line = re.sub(r"\b(inout|out)\s+(\w+)\s+(\w+)", r"\2& \3", line)
        line = re.sub(r"\bin\s+(\w+)\s+(\w+)", r"\1 \2", line)
        out_lines.append(line)
    return "\n".join(out_lines) + "\n"


def main():
    src, dst = sys.argv[1], sys.argv[2]
    os.makedirs(dst, exist_ok=True)
    for f in FILES:
        with open(os.path.join(src, f)) as fh:
            text = fh.read()
        base = os.path.basename(f)
        with open(os.path.join(dst, base.replace(".glsl", ".inc")), "w") as fh:
            fh.write(rewrite(text, base))


if __name__ == "__main__":
    main()
