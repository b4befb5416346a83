"""Static checks of bench.py and the package's Python modules on CPU.

A name that a function reads but that no scope defines (a local, an
argument, an enclosing function's variable, a module global or a builtin)
fails only when that line runs -- on a GPU, at the end of a long bench.  This
walks every function scope with `symtable` and fails on such names, the check
a linter's "undefined name" rule makes.
"""
import builtins
import os
import symtable

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FILES = ["bench.py", "__graft_entry__.py"] + [
    os.path.join("afepack_gb300", f) for f in sorted(os.listdir(os.path.join(ROOT, "afepack_gb300")))
    if f.endswith(".py")
]


def _module_names(top):
    names = set(dir(builtins)) | {"__file__", "__name__", "__doc__", "__spec__", "__builtins__", "__class__"}
    for s in top.get_symbols():
        if s.is_assigned() or s.is_imported() or s.is_namespace() or s.is_global():
            names.add(s.get_name())
    return names


def _undefined(table, module_names, enclosing=frozenset()):
    bad = []
    local = {s.get_name() for s in table.get_symbols()
             if s.is_assigned() or s.is_imported() or s.is_parameter() or s.is_namespace()}
    visible = enclosing | local if table.get_type() == "function" else enclosing
    for s in table.get_symbols():
        if not s.is_referenced():
            continue
        n = s.get_name()
        if s.is_global() or (table.get_type() == "function" and s.is_free()):
            if n not in module_names and n not in visible:
                bad.append((table.get_name(), table.get_lineno(), n))
    for child in table.get_children():
        bad += _undefined(child, module_names, visible)
    return bad


@pytest.mark.parametrize("rel", FILES)
def test_no_undefined_names(rel):
    src = open(os.path.join(ROOT, rel)).read()
    top = symtable.symtable(src, rel, "exec")
    mod = _module_names(top)
    bad = []
    for child in top.get_children():
        bad += _undefined(child, mod)
    assert not bad, f"{rel}: names read but defined nowhere: {bad}"


def test_checker_catches_a_stray_name():
    src = "def f(t):\n    a = t\n    return {'p50': lat}\n"
    top = symtable.symtable(src, "x.py", "exec")
    bad = []
    for child in top.get_children():
        bad += _undefined(child, _module_names(top))
    assert [b[2] for b in bad] == ["lat"]


def test_profiled_traffic_ratio_is_read_from_the_committed_summary():
    """bench.py's roofline `traffic` comes from the committed ncu summary of
    the batched sweep; a missing or unreadable line would silently report null."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    ratio = bench.profiled_ratio("poisson3d_p1_64", "rows_m_gs_batched")
    assert ratio is not None and 1.0 <= ratio <= 4.0


@pytest.mark.parametrize("name", sorted(f for f in os.listdir(os.path.join(ROOT, "profiles")) if f.endswith(".md")))
def test_profile_summaries_give_their_command(name):
    """Every ncu summary names the ncu command that made it, with
    --clock-control none, and runs committed files only."""
    text = open(os.path.join(ROOT, "profiles", name)).read()
    assert "ncu " in text and "--clock-control none" in text, name
    assert "_work/" not in text and "gpurun" not in text, name
