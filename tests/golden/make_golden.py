"""Writes the golden fixtures of the reference's own step-0 energy pins.

Run with the path of the reference tree (qusers/qsource) as the argument, or
in the environment variable QSOURCE_REFERENCE:

    python tests/golden/make_golden.py <reference tree>

For each pinned system it parses the reference's .top/.fep/.inp inputs with
qsource_gb300.system.System.from_files and stores the resulting start-up state
(0-based arrays) as <name>.npz next to this script.  golden.json records the
reference's published step-0 values for the same systems:

  basic_sph: tests/basic_tests/SPH_leap-frog_berendsen_benchmark.en row 1
             (QEL QVdW EL VdW QBND QANG QTOR QIMP BND ANG TOR IMP; lower == upper)
             with tests/basic_tests/prep_SPH inputs and the SPH substitutions of
             tests/basic_tests/run_test.sh:171-176
  test2:     tests/test2/eval_test.sh:67  "Q-surr. 1 1.0000 3.12 139.43"
  test3:     tests/test3/eval_test.sh:67  "Q-surr. 1 1.0000 -14.07 3.11"
  basic_sph_dynamics: rows 1-3 (step 0, step 50, final after 100 steps) of
             tests/basic_tests/SPH_{leap-frog,velocity-verlet}_{berendsen,
             langevin,nose-hoover}_benchmark.en
  basic_pbc: tests/basic_tests/PBC_leap-frog_berendsen_benchmark.en row 1 with
             tests/basic_tests/prep_PBC inputs and the PBC substitutions of
             tests/basic_tests/run_test.sh:177-181 (periodic box, q_atom 24,
             lrf 24)
  basic_pbc_dynamics: rows 1-3 of the six PBC_*_benchmark.en band files
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from qsource_gb300.system import System  # noqa: E402


def _read(p):
    with open(p) as f:
        return f.read()


def sph_inp(text: str) -> str:
    """The substitutions run_test.sh applies for the SPH leap-frog/Berendsen case."""
    return (text.replace("invalid-boundary", "[sphere]\nshell_radius\t16\nshell_force\t20")
            .replace("invalid-qatom", "q_atom\t99").replace("invalid-lrf", "lrf\t99")
            .replace("invalid-integrator", "leap-frog").replace("invalid-thermostat", "berendsen"))


def pbc_inp(text: str, integrator: str = "leap-frog", thermostat: str = "berendsen") -> str:
    """The substitutions run_test.sh applies for the PBC cases."""
    return (text.replace("invalid-boundary", "[PBC]\nput_solvent_back_in_box\ton\nput_solute_back_in_box\toff")
            .replace("invalid-qatom", "q_atom\t24").replace("invalid-lrf", "lrf\t24")
            .replace("invalid-integrator", integrator).replace("invalid-thermostat", thermostat))


def systems(ref: str):
    t = os.path.join(ref, "tests")
    yield "basic_sph", (_read(os.path.join(t, "basic_tests/prep_SPH/lig_w.top")),
                        _read(os.path.join(t, "basic_tests/prep_SPH/lig_w.fep")),
                        sph_inp(_read(os.path.join(t, "basic_tests/eq1.inp"))))
    yield "basic_pbc", (_read(os.path.join(t, "basic_tests/prep_PBC/lig_w.top")),
                        _read(os.path.join(t, "basic_tests/prep_PBC/lig_w.fep")),
                        pbc_inp(_read(os.path.join(t, "basic_tests/eq1.inp"))))
    for name in ("test2", "test3"):
        yield name, (_read(os.path.join(t, name, "prep/lig_w.top")), _read(os.path.join(t, name, "prep/lig_w.fep")),
                     _read(os.path.join(t, name, "eq1.inp")))


def parse_benchmark_row1(path: str) -> dict:
    cols = "QEL QVdW EL VdW QBND QANG QTOR QIMP BND ANG TOR IMP".split()
    with open(path) as f:
        for line in f:
            if line.startswith("1\t") or line.startswith("1 "):
                v = [float(x) for x in line.split()[1:]]
                return {c: v[2 * k] for k, c in enumerate(cols) if v[2 * k] == v[2 * k + 1]}
    raise ValueError(path)


def parse_benchmark_rows(path: str, nrows: int = 3) -> list:
    """Rows 1..nrows of a basic_tests band file: per row, the 15 columns
    QEL QVdW EL VdW QBND QANG QTOR QIMP BND ANG TOR IMP TOT KIN POT as
    [lower, upper] pairs."""
    cols = "QEL QVdW EL VdW QBND QANG QTOR QIMP BND ANG TOR IMP TOT KIN POT".split()
    out = []
    with open(path) as f:
        for line in f:
            if not line[:1].isdigit():
                continue
            v = [float(x) for x in line.split()[1:]]
            out.append({c: [v[2 * k], v[2 * k + 1]] for k, c in enumerate(cols)})
            if len(out) == nrows:
                break
    return out


def main(ref: str):
    gold = {}
    # rows 1-3 of the six sphere band files: step 0, step 50 and the final
    # energies after 100 steps of tests/basic_tests/eq1.inp
    gold["basic_sph_dynamics"] = {
        f"{integ}/{thermo}": parse_benchmark_rows(
            os.path.join(ref, f"tests/basic_tests/SPH_{integ}_{thermo}_benchmark.en"))
        for integ in ("leap-frog", "velocity-verlet") for thermo in ("berendsen", "langevin", "nose-hoover")}
    gold["basic_pbc_dynamics"] = {
        f"{integ}/{thermo}": parse_benchmark_rows(
            os.path.join(ref, f"tests/basic_tests/PBC_{integ}_{thermo}_benchmark.en"))
        for integ in ("leap-frog", "velocity-verlet") for thermo in ("berendsen", "langevin", "nose-hoover")}
    gold["basic_pbc"] = parse_benchmark_row1(os.path.join(ref, "tests/basic_tests/PBC_leap-frog_berendsen_benchmark.en"))
    for name, (top, fep, inp) in systems(ref):
        s = System.from_files(top, fep, inp)
        s.save_npz(os.path.join(HERE, f"{name}.npz"))
    gold["basic_sph"] = parse_benchmark_row1(os.path.join(ref, "tests/basic_tests/SPH_leap-frog_berendsen_benchmark.en"))
    for name in ("test2", "test3"):
        with open(os.path.join(ref, "tests", name, "eval_test.sh")) as f:
            for line in f:
                if line.startswith('INIT_QSURR_BM="Q-surr. 1 1.0000'):
                    el, vdw = line.split('"')[1].split()[3:5]
                    gold[name] = {"QEL": float(el), "QVdW": float(vdw)}
                    break
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(gold, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("QSOURCE_REFERENCE", "")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_golden.py <reference tree>  (or set QSOURCE_REFERENCE)")
    main(ref)
