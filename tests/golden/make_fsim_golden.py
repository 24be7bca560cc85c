"""Reference outputs for the fSim workload's parity cases, computed by the
unmodified reference built by oracle/Makefile (oracle/_ref/qflex_ref):

    python tests/golden/make_fsim_golden.py

  fsim_6x9_d4_region     6 x 9 grid with its disabled site, 4 fSim cycles
                         (bond 4), the workload's ordering (3 cuts x 2
                         values) with the last column as terminal region:
                         64 amplitudes of one string prefix
  fsim_6x9_d8_one_slice  the workload's circuit (8 cycles, bond 16), one
                         value per cut, no terminal region: one amplitude

Writes tests/golden/fsim_cases.json in the format of reference_cases.json.
"""
from __future__ import annotations

import json
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from qflex_gb300 import rqc  # noqa: E402
from tests.golden.make_golden import case  # noqa: E402


def main():
    cases = []
    c4, o4, g4, ini, finals = rqc.workload_c4()
    off = rqc.random_off_site(6, 9, 7)
    short = rqc.fsim_circuit(6, 9, 4, seed=0, off=[off])
    t = time.time()
    cases.append(case("fsim_6x9_d4_region", short, o4, g4, ini, finals[:1], memory="64GB", keep_gemms=False))
    print("fsim_6x9_d4_region", f"{time.time() - t:.1f} s", flush=True)
    one = rqc.ordering_6x9(off, cut_values=(1,), terminal_region=False)
    full = finals[1].replace("x", "0")
    t = time.time()
    cases.append(case("fsim_6x9_d8_one_slice", c4, one, g4, ini, [full], memory="64GB", keep_gemms=True))
    print("fsim_6x9_d8_one_slice", f"{time.time() - t:.1f} s", flush=True)
    path = Path(__file__).resolve().parent / "fsim_cases.json"
    path.write_text(json.dumps(cases))
    print("wrote", path)


if __name__ == "__main__":
    main()
