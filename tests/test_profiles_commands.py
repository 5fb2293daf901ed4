"""Every ncu summary under profiles/ names the command that made it, and
that command runs committed files only: a `bench.py` kernel or solver case
that exists, with flags that `bench.py` accepts.  (The summaries are text;
the cases and the flags are the reproducible part.)"""
import glob
import os
import re
import shlex
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _commands():
    out = []
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "*.txt"))):
        with open(path) as f:
            for line in f:
                m = re.match(r"#\s*command:\s*(.*)$", line.strip())
                if m:
                    out.append((os.path.basename(path), m.group(1)))
    return out


def test_every_summary_names_its_command():
    paths = sorted(glob.glob(os.path.join(ROOT, "profiles", "*.txt")))
    named = {p for p, _ in _commands()}
    assert paths and named == {os.path.basename(p) for p in paths}


def test_commands_use_existing_bench_cases_and_flags():
    with open(os.path.join(ROOT, "bench.py")) as f:
        parser_flags = set(re.findall(r'add_argument\("(--[a-z0-9-]+)"', f.read()))
    assert "--kernel-case" in parser_flags and "--solver-case" in parser_flags
    for name, cmd in _commands():
        for part in cmd.split("&&"):
            tok = shlex.split(part)
            if "bench.py" not in tok:
                continue
            args = tok[tok.index("bench.py") + 1:]
            for i, a in enumerate(args):
                if a.startswith("--"):
                    assert a in parser_flags, (name, a)
                if a == "--kernel-case":
                    assert args[i + 1] in bench.KERNEL_CASES, (name, args[i + 1])
                if a == "--solver-case":
                    assert args[i + 1] in bench.SOLVER_CASES, (name, args[i + 1])
            # the runs under ncu keep the clocks as the driver set them
            if tok[0] == "ncu":
                assert "--clock-control" in tok and tok[tok.index("--clock-control") + 1] == "none", name
