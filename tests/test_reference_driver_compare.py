"""The file comparison of the reference-driver run
(tests/reference_driver/run_reference_driver.py), on small Tecplot-like files
written here: byte equality, last-digit flips, and a column's scale taken
over a plot kind's files, so that a column holding round-off in one early
file (1e-17 far from the DNAPL) is measured on the values it takes later."""
import importlib.util
import pathlib

ROOT = pathlib.Path(__file__).resolve().parents[1]
spec = importlib.util.spec_from_file_location("rrd", ROOT / "tests" / "reference_driver" / "run_reference_driver.py")
rrd = importlib.util.module_from_spec(spec)
spec.loader.exec_module(rrd)


def write(p, rows, head='VARIABLES = "X","S2"'):
    p.write_text(head + "\n" + "\n".join(" ".join(r) for r in rows) + "\n")
    return p


def test_equal_files_and_digit_flips(tmp_path):
    a = write(tmp_path / "a.dat", [("0.1", "0.25"), ("0.2", "0.50")])
    b = write(tmp_path / "b.dat", [("0.1", "0.25"), ("0.2", "0.50")])
    assert rrd.compare(a, b) == {"equal": True}
    flip = write(tmp_path / "f.dat", [("0.1", "0.26"), ("0.2", "0.50")])  # one unit of the last digit
    r = rrd.compare(a, flip)
    assert not r["equal"] and r["last_digit_flips"] == 1 and r["max_rel"] == 0.0
    c = write(tmp_path / "c.dat", [("0.1", "0.25"), ("0.2", "0.60")])
    r = rrd.compare(a, c)
    assert r["beyond_one_digit"] == 1 and abs(r["max_rel"] - 0.1 / 0.5) < 1e-12


def test_round_off_column_measured_on_the_plot_kinds_scale(tmp_path):
    early_cpu = write(tmp_path / "e_cpu.dat", [("0.1", "4.8123e-17"), ("0.2", "1.0000e-18")])
    early_gpu = write(tmp_path / "e_gpu.dat", [("0.1", "4.7623e-17"), ("0.2", "1.0000e-18")])
    late_cpu = write(tmp_path / "l_cpu.dat", [("0.1", "0.4"), ("0.2", "0.3")])
    alone = rrd.compare(early_cpu, early_gpu)
    assert alone["max_rel"] > 1e-3  # the file's own column maximum is round-off
    scales = rrd.column_scales([early_cpu, late_cpu])
    assert scales[1] == 0.4 and scales[0] == 0.2
    r = rrd.compare(early_cpu, early_gpu, scales)
    assert not r["equal"] and r["max_rel"] < 1e-15
