"""The oracle is test infrastructure: the product never reaches it.

* No source of the package (webgraph-algo-rs_gb300/: the CUDA library, its
  host code and the Python mirror) imports, includes or calls oracle/.
* bench.py imports oracle/ only in its CPU legs: the reference arm, the
  functions that time the oracle, and the CPU-baseline blocks of the GPU
  arms, which run after the timed region and only without --no-cpu-baseline.
"""
import ast
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "webgraph-algo-rs_gb300")

ORACLE_REF = re.compile(r"(^\s*(from|import)\s+oracle\b)|(#\s*include\s*[<\"][^>\"]*oracle)|\bhbo_[a-z]"
                        r"|libhb_oracle", re.M)


def test_package_sources_do_not_reach_the_oracle():
    checked = 0
    for d, _, files in os.walk(PKG):
        if "_build" in d or "__pycache__" in d:
            continue
        for f in files:
            if f.endswith((".py", ".cpp", ".cu", ".h", ".cuh")):
                src = open(os.path.join(d, f), encoding="utf-8").read()
                m = ORACLE_REF.search(src)
                assert m is None, (os.path.join(d, f), m.group(0))
                checked += 1
    assert checked >= 10


CPU_LEGS = {"make_oracle_graph", "cpu_full_run", "cpu_bounded_run", "run_reference",
            "run_reference_visit", "run_reference_sumsweep"}


def _imports_oracle(node):
    if isinstance(node, ast.ImportFrom):
        return (node.module or "").split(".")[0] == "oracle"
    if isinstance(node, ast.Import):
        return any(a.name.split(".")[0] == "oracle" for a in node.names)
    return False


def test_bench_imports_the_oracle_only_in_its_cpu_legs():
    tree = ast.parse(open(os.path.join(ROOT, "bench.py"), encoding="utf-8").read())
    assert not any(_imports_oracle(n) for n in tree.body), "module-level oracle import"
    found = 0
    for fn in (n for n in tree.body if isinstance(n, ast.FunctionDef)):
        # the guard of each import: the innermost `if` around it
        parents = {}
        for p in ast.walk(fn):
            for c in ast.iter_child_nodes(p):
                parents[c] = p
        for node in ast.walk(fn):
            if not _imports_oracle(node):
                continue
            found += 1
            if fn.name in CPU_LEGS:
                continue
            guard = parents.get(node)
            while guard is not None and not isinstance(guard, ast.If):
                guard = parents.get(guard)
            assert guard is not None and "no_cpu_baseline" in ast.unparse(guard.test), \
                (fn.name, node.lineno)
    assert found >= 5
