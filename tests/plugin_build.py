"""Builds the library with the test-only heat plugin (tests/plugins/heat.cu)
linked in, as a separate shared library next to the default one."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEAT = os.path.join(ROOT, "tests", "plugins", "heat.cu")
HEAT_LIB = os.path.join(ROOT, "bsam1.2_gb300", "_build", "libbsamg_heat.so")


def build_heat():
    import __graft_entry__ as ge
    return ge._load_build_module().build(extra_plugins=[HEAT], lib=HEAT_LIB)


def run_with_heat(code, timeout=600):
    """Run python code in a fresh process whose package loads the heat build."""
    env = dict(os.environ, BSAMG_LIBRARY=build_heat())
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=timeout)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout
