"""TEST INFRASTRUCTURE: rewrites the reference's compute shaders into C++ that compiles against
oracle/ref/glsl_shim.hpp, so the reference's own shader code can run on the CPU and pin the oracle.

Reads assets/shaders/voxelShared.comp + voxelLighting.comp / voxelDraw.comp from the reference tree
and writes oracle/_ref/shader_light.inc and oracle/_ref/shader_draw.inc (generated, not committed).
Only the constructs C++ does not accept are rewritten; expressions and statements are kept as they are:
  * `#version`, `#line` and `layout(local_size...) in;` lines are dropped;
  * storage-buffer blocks become gbuf<T> globals, `layout(...) uniform image2D` an image2D global,
    and the `uniform` qualifier is dropped (uniforms become globals the harness sets);
  * `inout T x` / `out T x` parameters become `T& x`;
  * swizzles (.xyz, .yzx, ...) become calls (.xyz(), ...);
  * floating literals get an `f` suffix (GLSL literals are single precision);
  * a local variable named like the bitCount() built-in is renamed;
  * main() becomes shader_main(); a reset_globals() restores the initialised globals that GLSL
    re-initialises for every invocation;
  * the draw's `float finalDepth;` is initialised to -1 (the shader leaves it undefined when the ray
    misses the map's bounding box);
  * a capture call is placed after the lighting shader clamps its results, before it quantises them.

    python oracle/ref/glsl_to_cpp.py REFERENCE_ROOT OUT_DIR
"""
import os
import re
import sys


def translate(src, capture=False, kind=""):
    out_lines = []
    for ln in src.splitlines():
        s = ln.strip()
        if s.startswith("#version") or s.startswith("#line"):
            continue
        if re.match(r"layout\s*\(\s*local_size", s):
            continue
        out_lines.append(ln)
    src = "\n".join(out_lines)
    # storage buffers: layout(...) restrict [readonly] buffer Name { T field[]; };
    src = re.sub(r"layout\s*\([^)]*\)\s*(?:restrict\s+)?(?:readonly\s+)?buffer\s+\w+\s*\{\s*(\w+)\s+(\w+)\s*\[\s*\d*\s*\]\s*;[^}]*\}\s*;",
                 r"gbuf<\1> \2;", src, flags=re.S)
    src = re.sub(r"layout\s*\([^)]*\)\s*uniform\s+image2D\s+(\w+)\s*;", r"image2D \1;", src)
    src = re.sub(r"\buniform\s+", "", src)
    src = re.sub(r"\b(inout|out)\s+(\w+)\s+(\w+)", r"\2& \3", src)
    src = re.sub(r"\.([xyzw]{2,4})\b", r".\1()", src)
    src = re.sub(r"(?<![\w.])(\d+\.\d*|\.\d+)([eE][+-]?\d+)?(?![\w.])", r"\1\2f", src)
    src = re.sub(r"uint\s+bitCount\s*=\s*bitCount\s*\(", "uint bitCount_ = bitCount(", src)
    src = re.sub(r"\bbitCount\b(?!\s*\()", "bitCount_", src)
    src = re.sub(r"\bvoid\s+main\s*\(\s*\)", "void shader_main()", src)
    if kind == "draw":
        src = re.sub(r"\bfloat\s+finalDepth\s*;", "float finalDepth = -1.0f;", src)
    if capture:
        src, n = re.subn(r"(diffuseLight\s*=\s*clamp\(diffuseLight,[^;]*;)", r"\1\n\tpin_capture(voxelIndex, specLight, diffuseLight);", src)
        assert n == 1, "capture point not found"
    # initialised globals, re-initialised per invocation
    resets = []
    depth = 0
    for ln in src.splitlines():
        if depth == 0:
            m = re.match(r"^\s*(bool|uint|int|float|vec3)\s+(\w+)\s*=\s*([^;]+);", ln)
            if m:
                resets.append("%s = %s;" % (m.group(2), m.group(3)))
        depth += ln.count("{") - ln.count("}")
    macros = re.findall(r"^\s*#define\s+(\w+)", src, flags=re.M)
    body = ["using namespace glsl;", src, "void reset_globals() { " + " ".join(resets) + " }"]
    body += ["#undef %s" % m for m in macros]
    return "\n".join(body) + "\n"


def main():
    ref, out = sys.argv[1], sys.argv[2]
    d = os.path.join(ref, "assets", "shaders")
    shared = open(os.path.join(d, "voxelShared.comp")).read()
    os.makedirs(out, exist_ok=True)
    for name, fn, cap in (("light", "voxelLighting.comp", True), ("draw", "voxelDraw.comp", False)):
        main_src = open(os.path.join(d, fn)).read()
        # the reference's loader places the shared source after the #version line (shader.c:185-231)
        txt = translate(shared + "\n" + main_src, capture=cap, kind=name)
        with open(os.path.join(out, "shader_%s.inc" % name), "w") as f:
            f.write(txt)


if __name__ == "__main__":
    main()
