"""The entry scripts compile (a syntax error there would only show on the GPU machine)."""
import py_compile
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_entry_scripts_compile():
    for name in ("bench.py", "__graft_entry__.py"):
        py_compile.compile(str(ROOT / name), doraise=True)
