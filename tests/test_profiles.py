"""The ncu summaries under profiles/ cite the command that produced them; every such command
must run committed files only: bench.py with options its parser accepts."""
import glob
import os
import re
import shlex

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SUMMARIES = sorted(glob.glob(os.path.join(ROOT, "profiles", "*.md")) + glob.glob(os.path.join(ROOT, "profiles", "*.txt")))


def _commands(text: str):
    """The indented command block of a summary, continuation lines joined, split at &&."""
    block = []
    for line in text.splitlines():
        if line.startswith("    ") and line.strip():
            block.append(line.strip().rstrip("\\").strip())
        elif block:
            break
    for part in " ".join(block).split("&&"):
        if part.strip():
            yield shlex.split(part.strip())


def test_profiles_present():
    assert SUMMARIES, "no ncu summaries committed"


@pytest.mark.parametrize("path", SUMMARIES, ids=[os.path.basename(p) for p in SUMMARIES])
def test_profile_commands_use_committed_entry_points(path):
    import bench
    text = open(path).read()
    cmds = list(_commands(text))
    assert cmds, f"{path}: no command block"
    for argv in cmds:
        if argv[0] == "ncu":
            assert "--clock-control" in argv and argv[argv.index("--clock-control") + 1] == "none", argv
            i = argv.index("python")
            argv = argv[i:]
        assert argv[:2] == ["python", "bench.py"], argv
        bench.make_parser().parse_args(argv[2:])   # exits (SystemExit) on an unknown option
    # no raw report or other binary output is committed next to the summaries
    assert not re.search(r"\.ncu-rep\b", os.path.basename(path))
