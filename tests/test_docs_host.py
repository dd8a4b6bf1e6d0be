"""The Python examples of INTEGRATION.md stay valid against the package (no
GPU): every block parses, and every name a block imports from ocelot_gb300
exists there."""
import ast
import importlib
import os
import re

import pytest

from conftest import REPO


def _blocks():
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    return re.findall(r"```python\n(.*?)```", text, re.S)


def test_there_are_examples():
    assert len(_blocks()) >= 5


@pytest.mark.parametrize("i", range(len(_blocks())))
def test_example_parses_and_its_imports_exist(i):
    tree = ast.parse(_blocks()[i])
    for node in ast.walk(tree):
        if isinstance(node, ast.ImportFrom) and node.module and node.module.split(".")[0] == "ocelot_gb300":
            mod = importlib.import_module(node.module)
            for alias in node.names:
                if not hasattr(mod, alias.name):   # a submodule, which the statement imports
                    importlib.import_module(f"{node.module}.{alias.name}")
        elif isinstance(node, ast.Import):
            for alias in node.names:
                if alias.name.split(".")[0] == "ocelot_gb300":
                    importlib.import_module(alias.name)
