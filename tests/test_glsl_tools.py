"""The GLSL -> C++ conversion that lets the reference shaders compile unchanged on glm
(oracle/ref/glsl_to_cpp.py): only the five mechanical changes it documents, nothing else."""
import importlib.util
import os

from conftest import REPO


def _convert():
    spec = importlib.util.spec_from_file_location("glsl_to_cpp", os.path.join(REPO, "oracle", "ref", "glsl_to_cpp.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.convert


SHADER = """#version 450
#extension GL_ARB_separate_shader_objects : enable
precision highp float;
layout(location = 0) in vec2 fragUV;
layout(location = 0) out vec4 outColor;
#define SCALE 0.5 // half
float f(in vec3 p, inout float c) {
    vec3 q = p.xyz * 2.0 + vec3(1e-3, .25, 3.);
    c = 1.5e2;
    q.xy = p.zx;
    q.rgb *= 0.5;
    return dot(q.xyz, p) + q.x + 10;  // 2.0 in a comment stays
}
"""


def test_glsl_only_lines_are_dropped():
    out = _convert()(SHADER)
    assert out.startswith('#include "glsl_shim.h"\n')
    for s in ("#version 450", "#extension", "precision highp float;"):
        line = next(l for l in out.splitlines() if s in l)
        assert line.startswith("// (GLSL only)")


def test_float_literals_get_the_float_suffix():
    out = _convert()(SHADER)
    assert "#define SCALE 0.5f // half" in out
    assert "p.xyz() * 2.0f + vec3(1e-3f, .25f, 3.f)" in out
    assert "c = 1.5e2f;" in out
    assert "+ 10;" in out                 # integer literals stay integers
    assert "// 2.0 in a comment stays" in out


def test_swizzle_reads_get_the_call_form_and_writes_do_not():
    out = _convert()(SHADER)
    assert "q.xy = p.zx();" in out        # written swizzle kept, read swizzle called
    assert "q.rgb *= 0.5f;" in out        # compound assignment to a swizzle kept
    assert "dot(q.xyz(), p) + q.x" in out  # single components are plain members


def test_stage_variables_become_thread_local():
    out = _convert()(SHADER)
    assert "thread_local vec2 fragUV;" in out
    assert "thread_local vec4 outColor;" in out
    assert "float f(in vec3 p, inout float c)" in out  # parameter qualifiers are left to the shim
