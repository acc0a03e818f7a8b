"""The CLI's flag contract against the reference binary itself.

oracle/ref_build.sh compiles the reference's unmodified sources into oracle/_ref/procell_ref
(here, where the sources are mounted, or on a GPU machine from the staged copy). Its argument
handling (src/io/cmdargs.cpp:11-375) and its ratio-sum check (src/io/parser.cu:46-66) run
before any CUDA call, so both binaries can be compared on a machine without a GPU. Skipped
when the reference binary has not been built.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, "oracle", "_ref", "procell_ref")

pytestmark = pytest.mark.skipif(not os.path.exists(REF), reason="reference binary not built")

SAME = [
    ["-x"], ["-h"], ["-h", "a", "-h", "b"], ["--histogram", "a", "-h", "b"], ["-c"],
    ["-c", "a", "--cell-types", "b"], ["-o"], ["-o", "a", "--output-histogram", "b"],
    ["-t", "-3"], ["-t"], ["-t", "1", "--time-max", "2"], ["-p", "0"], ["-p", "-1"], ["-p"],
    ["-p", "abc"], ["-p", "1", "-p", "2"], ["-d", "0"], ["-d", "24"], ["-d", "abc"], ["-d"],
    ["-d", "3", "-d", "4"], ["-r", "-r"], ["--track-ratio", "-r"], ["positional"],
    ["-h", "a", "extra"], ["--help"],
]


def run(binary, args, cwd):
    return subprocess.run([binary, *args], capture_output=True, text=True, cwd=cwd, timeout=60)


@pytest.mark.parametrize("args", SAME, ids=[" ".join(a) or "none" for a in SAME])
def test_same_messages_and_exit_codes(built, tmp_path, args):
    from procell import _lib
    ref = run(REF, args, tmp_path)
    ours = run(_lib.CLI_PATH, args, tmp_path)
    assert ours.returncode == ref.returncode
    if args == ["--help"]:
        return  # the reference prints a placeholder; ours prints usage (both exit 0)
    assert ours.stdout == ref.stdout


def test_missing_arguments_except_phi(built, tmp_path):
    from procell import _lib
    # the reference also lists --phi-min (-p); here -p is optional (automatic threshold)
    ref = run(REF, ["-t", "1"], tmp_path)
    ours = run(_lib.CLI_PATH, ["-t", "1"], tmp_path)
    assert ref.returncode == ours.returncode == 1
    assert ours.stdout == ref.stdout.replace("--phi-min (-p)\n", "")


def test_ratio_sum_error(built, tmp_path):
    from procell import _lib
    (tmp_path / "h.txt").write_text("4 10\n")
    (tmp_path / "c.txt").write_text("0.5 10 1\n0.4 20 1\n")
    args = ["-h", "h.txt", "-c", "c.txt", "-t", "1", "-p", "1"]
    ref = run(REF, args, tmp_path)
    ours = run(_lib.CLI_PATH, args, tmp_path)
    assert ref.returncode == ours.returncode == 1
    assert ours.stdout == ref.stdout
