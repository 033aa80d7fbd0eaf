"""The drop-in CLIs report bad arguments and bad .tri inputs as the reference does:
the same lines on stdout and exit status 0 (main.cpp:100-196, 244-267; tri_tools.h:75-115;
partitioner.cpp:12-28).  Every case stops before the build, or at the partition count;
without a GPU the build that follows fails cleanly."""
import json
import os
import subprocess

import pytest

import cli_cases
import ooc_svo_builder_gb300 as ooc
import pyoracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "cli_messages.json")
BIN = os.path.join(os.path.dirname(ooc.LIB_PATH), "bin")
EXPECTED = json.load(open(GOLDEN))


@pytest.fixture(scope="module")
def inputs(tmp_path_factory):
    d = str(tmp_path_factory.mktemp("cli"))
    cli_cases.make_inputs(d)
    return d


def run(folder, exe, args, path):
    return subprocess.run([os.path.join(path, exe), *args], cwd=folder, stdout=subprocess.PIPE, text=True,
                          timeout=300)


def test_every_case_has_a_recorded_answer():
    assert sorted(EXPECTED) == sorted(cli_cases.case_id(e, a) for e, a in cli_cases.CASES)


@pytest.mark.parametrize("exe,args", cli_cases.CASES, ids=[cli_cases.case_id(e, a) for e, a in cli_cases.CASES])
def test_cli_diagnostics_match_reference(inputs, exe, args):
    want = EXPECTED[cli_cases.case_id(exe, args)]
    r = run(inputs, exe, args, BIN)
    assert r.returncode == want["status"] == 0
    assert cli_cases.diagnostics(r.stdout) == want["lines"]


@pytest.mark.parametrize("exe,args", cli_cases.CASES[:6], ids=[cli_cases.case_id(e, a) for e, a in cli_cases.CASES[:6]])
def test_recorded_answers_are_the_reference_build(inputs, exe, args):
    """Where the reference build is present, the recorded lines are still its lines."""
    ref = os.path.dirname(pyoracle.ref_binary(True))
    if not os.path.exists(os.path.join(ref, exe)):
        pytest.skip("reference build not present (make -C oracle ref needs the reference sources)")
    r = run(inputs, exe, args, ref)
    assert cli_cases.diagnostics(r.stdout) == EXPECTED[cli_cases.case_id(exe, args)]["lines"]


FULL = json.load(open(os.path.join(os.path.dirname(GOLDEN), "cli_full_runs.json")))


def test_every_complete_run_has_a_recorded_answer():
    assert sorted(FULL) == sorted(cli_cases.case_id(e, a) for e, a in cli_cases.FULL_RUNS)


@pytest.mark.parametrize("exe,args", cli_cases.FULL_RUNS, ids=[cli_cases.case_id(e, a) for e, a in cli_cases.FULL_RUNS])
def test_recorded_complete_runs_are_the_reference_build(inputs, exe, args):
    """Where the reference build is present, the recorded complete runs are still its output."""
    ref = os.path.dirname(pyoracle.ref_binary(True))
    if not os.path.exists(os.path.join(ref, exe)):
        pytest.skip("reference build not present (make -C oracle ref needs the reference sources)")
    r = run(inputs, exe, args, ref)
    assert cli_cases.full_run_lines(r.stdout) == FULL[cli_cases.case_id(exe, args)]["lines"]
