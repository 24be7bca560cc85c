"""The C++ drop-in (include/qflex_gb300_evaluate.hpp) and the command-line
front end (qflex_gb300/qflex), run the way a reference user runs them.

The C++ program tests/cpp/evaluate_circuit_dropin.cpp is compiled against
the header and the library: its input-model checks need no GPU; its
EvaluateCircuit checks are the reference's known-answer test
(tests/src/evaluate_circuit_test.cpp:185-207). The CLI is checked for its
output lines and exit codes (src/main.cpp:140-155: 1 for std::exception,
2 for a thrown error message)."""
import subprocess

import pytest

from tests.conftest import ROOT

CLI = ROOT / "qflex_gb300" / "qflex"


@pytest.fixture(scope="module")
def dropin(built_lib, tmp_path_factory):
    exe = tmp_path_factory.mktemp("dropin") / "evaluate_circuit_dropin"
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", str(ROOT / "include"),
                    str(ROOT / "tests" / "cpp" / "evaluate_circuit_dropin.cpp"), "-L", str(built_lib.parent),
                    "-lqflex_gb300", f"-Wl,-rpath,{built_lib.parent}", "-o", str(exe)], check=True,
                   capture_output=True, text=True)
    return exe


def _run(exe, mode):
    out = subprocess.run([str(exe), mode], capture_output=True, text=True, timeout=600)
    fails = [ln for ln in out.stdout.splitlines() if not ln.startswith("OK ")]
    return out, fails


def test_cpp_input_models(dropin):
    """QflexCircuit / QflexGrid / QflexOrdering expose the reference's parsed
    members, round-trip through text, and throw the reference's errors at
    load time; EvaluateCircuit(nullptr) throws."""
    out, fails = _run(dropin, "parse")
    assert out.returncode == 0 and not fails, out.stdout + out.stderr
    assert out.stdout.count("OK ") == 13


@pytest.mark.gpu
def test_cpp_evaluate_circuit_known_answer(dropin):
    out, fails = _run(dropin, "eval")
    assert out.returncode == 0 and not fails, out.stdout + out.stderr
    assert out.stdout.count("OK ") == 7


def _files(tmp_path, ref_cases):
    case = ref_cases["simple"]
    paths = []
    for name in ("circuit", "ordering", "grid"):
        p = tmp_path / name
        p.write_text(case[name])
        paths.append(str(p))
    return paths


def test_cli_usage_and_std_exception_exit_codes(built_lib, tmp_path, ref_cases):
    out = subprocess.run([str(CLI)], capture_output=True, text=True)
    assert out.returncode == 1 and "Usage:" in out.stderr
    c, o, g = _files(tmp_path, ref_cases)
    # A memory limit that does not fit in 64 bits: std::out_of_range, exit 1.
    out = subprocess.run([str(CLI), "-c", c, "-o", o, "-g", g, "--memory=99999999999999999999999GB"],
                         capture_output=True, text=True)
    assert out.returncode == 1 and out.stdout == ""
    # A missing input file: the reference's thrown message, exit 2.
    out = subprocess.run([str(CLI), str(tmp_path / "missing"), o, g], capture_output=True, text=True)
    assert out.returncode == 2 and "Cannot open circuit file" in out.stderr


@pytest.mark.gpu
def test_cli_known_answer_and_errors(built_lib, tmp_path, ref_cases):
    c, o, g = _files(tmp_path, ref_cases)
    out = subprocess.run([str(CLI), c, o, g, "00000", "1100x"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.splitlines()
    assert [ln.split(":")[0] for ln in lines] == ["00000 --> 11000", "00000 --> 11001"]
    amps = [complex(*map(float, ln.split(": ")[1].split())) for ln in lines]
    assert abs(amps[0] - (0.10669 + 0.04419j)) < 2e-5 and abs(amps[1] - (-0.01831 - 0.25758j)) < 2e-5
    # The same through the -c/-o/-g form and the complex128 oracle.
    out = subprocess.run([str(CLI), "-c", c, "-o", o, "-g", g, "--initial-conf=00000", "--final-conf=1100x",
                          "--precision=fp64"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.splitlines()[0].startswith("00000 --> 11000: 0.1066")
    # The reference's memory-limit error, wrapped as its main() wraps it: exit 2.
    out = subprocess.run([str(CLI), c, o, g, "00000", "1100x", "0", "512B"], capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 2 and out.stdout == ""
    assert "Failed to call EvaluateCircuit()" in out.stderr and "exceeds memory limit" in out.stderr


def test_simulate_option_handling_matches_pybind(built_lib, ref_cases, tmp_path, capsys):
    """qflex.simulate's option handling (src/pybind_main.cpp:26-138), on a
    planning-only context: every malformed option prints the reference's
    message and returns []; the data keys load in the order grid, circuit,
    ordering, so the first bad one is the one reported; the memory limit is
    global state as there; a valid call returns the reference's output
    states."""
    from qflex_gb300 import Context
    from qflex_gb300.qflex import simulate

    ctx = Context(-1)
    case = ref_cases["simple"]
    base = {"circuit": case["circuit"].splitlines(), "ordering": case["ordering"].splitlines(),
            "grid": case["grid"].splitlines(), "initial_state": "00000", "final_state": "1100x"}

    out = simulate(dict(base), context=ctx)
    assert [s for s, _ in out] == ["11000", "11001"]
    assert [s for s, _ in simulate(dict(base, memory_limit="16GB"), context=ctx)] == ["11000", "11001"]
    capsys.readouterr()

    def message(options):
        assert simulate(options, context=ctx) == []
        return capsys.readouterr().err

    assert "'circuit' must be a list of strings." in message(dict(base, circuit=5))
    no_grid = {k: v for k, v in base.items() if k != "grid"}
    assert "'grid_filename' must be a string." in message(dict(no_grid, grid_filename=3))
    # grid loads first: with both malformed, the grid is reported
    assert "'grid' must be a list of strings." in message(dict(base, grid=1, circuit=5))
    assert "Not yet supported" in message(dict(base, final_states=["1100x", "0000x"]))
    assert "states must be strings." in message(dict(base, initial_states=["00000", 7]))
    assert "final_states must be a list of strings." in message(dict(base, final_states=7))
    assert "states must be strings." in message(dict(base, final_state=7))
    assert "'memory_limit' must be positive." in message(dict(base, memory_limit=0))
    no_circuit = {k: v for k, v in base.items() if k != "circuit"}
    missing = tmp_path / "missing.txt"
    assert f"Cannot open circuit file {missing}." in message(dict(no_circuit, circuit_filename=str(missing)))
    assert "exceeds memory limit" in message(dict(base, memory_limit=64))
    # A memory_limit of another type is not an error there (the message is
    # built but not thrown): the limit is global state and keeps the
    # previous call's value, here 64 bytes, then 16 GB.
    assert "exceeds memory limit" in message(dict(base, memory_limit=1.5))
    simulate(dict(base, memory_limit="16GB"), context=ctx)
    assert [s for s, _ in simulate(dict(base, memory_limit=1.5), context=ctx)] == ["11000", "11001"]
    # Without the key the limit returns to the 1 GiB default.
    assert [s for s, _ in simulate(dict(base), context=ctx)] == ["11000", "11001"]


def test_cli_argument_errors(built_lib, tmp_path):
    """The CLI's failures before any evaluation (no GPU needed): missing
    arguments print the usage with exit code 1; an unknown precision and an
    unreadable input file are error messages, exit code 2, as the reference's
    main.cpp returns for a thrown message (src/main.cpp:148-155)."""
    assert CLI.exists()
    usage = subprocess.run([str(CLI)], capture_output=True, text=True, timeout=60)
    assert usage.returncode == 1 and "qflex" in usage.stderr.lower()
    for name in ("c.txt", "o.txt", "g.txt"):
        (tmp_path / name).write_text("1 1\n" if name == "g.txt" else "")
    args = ["-c", str(tmp_path / "c.txt"), "-o", str(tmp_path / "o.txt"), "-g", str(tmp_path / "g.txt")]
    bad = subprocess.run([str(CLI), *args, "--precision=fp8"], capture_output=True, text=True, timeout=60)
    assert bad.returncode == 2 and "Unknown precision fp8" in bad.stderr
    missing = tmp_path / "none.txt"
    args[1] = str(missing)
    gone = subprocess.run([str(CLI), *args], capture_output=True, text=True, timeout=60)
    assert gone.returncode == 2 and f"Cannot open circuit file {missing}" in gone.stderr
