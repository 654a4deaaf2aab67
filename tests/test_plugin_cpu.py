"""The device plugin interface (no GPU needed): the library's problems are
plugins found by name, and a plugin file kept outside the library (the
test-only tests/plugins/heat.cu) links into a build of its own and registers
there without any library source changing."""
import pytest

from tests.plugin_build import run_with_heat


def test_shipped_plugins_are_registered(pkg):
    api = pkg.api
    assert [api.problem_kind(n) for n in ("ch", "biogrowth", "growth")] == [1, 2, 3]
    assert api.problem_info("ch") == (2, 2, True)
    assert api.problem_info("biogrowth") == (2, 5, False)
    assert api.problem_info("growth") == (3, 6, True)
    with pytest.raises(pkg.BsamgError):
        api.problem_kind("heat")  # only in the test build


def test_a_plugin_outside_the_library_registers():
    out = run_with_heat(
        "import __graft_entry__ as ge\n"
        "api = ge.load_package().api\n"
        "print(api.problem_kind('heat'), *api.problem_info('heat'), api.problem_kind('ch'))\n")
    assert out.split() == ["40", "2", "2", "True", "1"]
