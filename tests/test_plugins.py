"""The ufo-core plugin shells (plugins/): they compile, as C11 with every
warning an error, against declarations of the glib / GObject / ufo-core API
they use (tests/plugin_stubs; the libraries themselves are absent here),
and each exports the constructor ufo-core's plugin manager looks up for
its node name (ufo_ir_<name>_task_new, src/tasks/ufo-ir-sart-task.c:146-150
in the reference) with the reference's property names."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PLUGINS = os.path.join(ROOT, "plugins")
NODES = {
    "parallel-projector": ["model", "angles_num", "is_forward", "axis_position", "step", "relaxation",
                           "correction_scale"],
    "sart": ["num-iterations", "projector", "relaxation_factor"],
    "sirt": ["num-iterations", "projector", "relaxation_factor"],
    "asdpocs": ["num-iterations", "projector", "beta", "beta_red", "ng", "alpha", "alpha_red", "r_max",
                "positive_constraint", "df_minimizer"],
    "sbtv": ["num-iterations", "projector", "lambda", "mu"],
}


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
@pytest.mark.parametrize("src", sorted(f for f in os.listdir(PLUGINS) if f.endswith(".c")))
def test_plugin_shell_compiles(src):
    out = subprocess.run(["gcc", "-std=c11", "-fsyntax-only", "-Wall", "-Wextra", "-Wno-unused-parameter",
                          "-Werror", "-I", os.path.join(ROOT, "tests", "plugin_stubs"),
                          "-I", os.path.join(ROOT, "include"), "-I", PLUGINS, os.path.join(PLUGINS, src)],
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr


@pytest.mark.parametrize("node", sorted(NODES))
def test_plugin_shell_constructor_and_properties(node):
    src = open(os.path.join(PLUGINS, f"ufo-ir-{node}-task.c")).read()
    if node != "parallel-projector":
        src += open(os.path.join(PLUGINS, "ufo-ir-method-shell.h")).read()
    ctor = "ufo_ir_" + node.replace("-", "_") + "_task_new"
    assert re.search(r"^UfoNode \*\n" + ctor + r" \(void\)", src, re.M), ctor
    names = re.findall(r'g_param_spec_\w+ \("([\w-]+)"', src)
    for prop in NODES[node]:
        assert prop in names, (node, prop)
    cmake = open(os.path.join(PLUGINS, "CMakeLists.txt")).read()
    assert node in cmake
