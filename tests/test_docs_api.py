"""The user-facing documents name only what exists (CPU): every ``from mlpcg_gb300... import``
in their Python blocks resolves, and every C entry point they mention is declared in the header."""
import importlib
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
DOCS = ["README.md", "INTEGRATION.md"]


def _python_blocks(text):
    return re.findall(r"```python\n(.*?)```", text, flags=re.S)


@pytest.mark.parametrize("doc", DOCS)
def test_documented_python_names_exist(doc):
    text = (ROOT / doc).read_text()
    checked = 0
    for block in _python_blocks(text):
        for mod, names in re.findall(r"^\s*from (mlpcg_gb300(?:\.\w+)*) import ([\w, ]+)", block, flags=re.M):
            m = importlib.import_module(mod)
            for name in (n.strip() for n in names.split(",")):
                assert hasattr(m, name) or importlib.util.find_spec(f"{mod}.{name}") is not None, \
                    f"{doc}: {mod}.{name} does not exist"
                checked += 1
    assert checked > 0


@pytest.mark.parametrize("doc", ["INTEGRATION.md", "DESIGN.md"])
def test_documented_c_entry_points_are_declared(doc):
    header = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "mlpcg_gb300.h").read_text(), flags=re.S)
    declared = set(re.findall(r"\b(mlpcg_[a-z0-9_]+)\s*\(", header))
    mentioned = set(re.findall(r"`(mlpcg_[a-z0-9_]+)(?:\(|`)", (ROOT / doc).read_text()))
    assert mentioned, doc
    unknown = {m for m in mentioned if m not in declared and not m.startswith("mlpcg_gb300")}
    assert not unknown, f"{doc} names undeclared entry points: {sorted(unknown)}"
