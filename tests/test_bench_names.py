"""Static check of bench.py and __graft_entry__.py: every name a top-level
function loads is a builtin, a module-level name, or bound in that function
(parameters, assignments, imports).  The GPU paths of these scripts only run
on a device, so a name used without its import would otherwise surface
there first."""
import ast
import builtins
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _undefined(path):
    tree = ast.parse(open(path).read())
    glob = set(dir(builtins))
    for n in tree.body:
        if isinstance(n, (ast.FunctionDef, ast.ClassDef)):
            glob.add(n.name)
        elif isinstance(n, (ast.Import, ast.ImportFrom)):
            glob.update((a.asname or a.name).split(".")[0] for a in n.names)
        elif isinstance(n, (ast.Assign, ast.AnnAssign)):
            for t in (n.targets if isinstance(n, ast.Assign) else [n.target]):
                glob.update(x.id for x in ast.walk(t) if isinstance(x, ast.Name))
    missing = []
    for f in tree.body:
        if not isinstance(f, ast.FunctionDef):
            continue
        bound = set()
        for x in ast.walk(f):
            if isinstance(x, ast.arg):
                bound.add(x.arg)
            elif isinstance(x, ast.Name) and isinstance(x.ctx, (ast.Store, ast.Del)):
                bound.add(x.id)
            elif isinstance(x, (ast.Import, ast.ImportFrom)):
                bound.update((a.asname or a.name).split(".")[0] for a in x.names)
            elif isinstance(x, (ast.FunctionDef, ast.ClassDef)) and x is not f:
                bound.add(x.name)
            elif isinstance(x, ast.ExceptHandler) and x.name:
                bound.add(x.name)
        missing += ["%s:%d %s in %s()" % (os.path.basename(path), x.lineno, x.id, f.name)
                    for x in ast.walk(f)
                    if isinstance(x, ast.Name) and isinstance(x.ctx, ast.Load)
                    and x.id not in bound and x.id not in glob]
    return missing


@pytest.mark.parametrize("name", ["bench.py", "__graft_entry__.py"])
def test_no_undefined_names(name):
    assert _undefined(os.path.join(ROOT, name)) == []
