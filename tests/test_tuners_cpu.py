"""The tuners write the tables the library compiles against (lagrbf_gb300/csrc/lgb_factor_tune.h,
lgb_eval_tune.h).  Driven here with synthetic timings instead of GPU measurements: the fastest
candidate goes into the table, and the written header compiles with the library's own macros."""
import os
import subprocess
import sys

from lagrbf_gb300 import tune_eval, tune_factor

CSRC = os.path.join(os.path.dirname(tune_eval.__file__), "csrc")


def _compiles(tmp_path, header_dir, header_name, body):
    """Compiles a C unit that includes the library's internal header, then the table."""
    src = tmp_path / "use.c"
    src.write_text('#include "lgb_internal.h"\n#include "%s"\n%s\n' % (header_name, body))
    cuda = "/usr/local/cuda/include"
    r = subprocess.run(["gcc", "-std=gnu11", "-c", "-I", str(header_dir), "-I", CSRC, "-I", cuda, str(src),
                        "-o", str(tmp_path / "use.o")], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    return r.returncode, r.stdout


def test_eval_tuner_picks_the_fastest_ring(tmp_path, monkeypatch):
    built, state = [], {"nb": None}
    times = {(nb, b): 30.0 - nb - b / 1000.0 for nb in tune_eval.STAGES for b in tune_eval.BUDGETS}
    times[(3, 1536)] = 10.0

    def fake_build(flags):
        built.append(flags)
        if flags:
            state["nb"] = int(flags.split("=")[1])

    monkeypatch.setattr(tune_eval, "build", fake_build)
    monkeypatch.setattr(tune_eval, "measure", lambda b, np_: times[(state["nb"], b)])
    out = tmp_path / "lgb_eval_tune.h"
    monkeypatch.setattr(sys, "argv", ["tune_eval", "--np", "1000", "--out", str(out)])
    tune_eval.main()
    text = out.read_text()
    assert "#define LGB_EVR_NB_TUNED 3" in text and "#define LGB_TMA_BUDGET_TUNED 1536" in text
    assert built[-1] == ""  # the library is rebuilt without tuning flags at the end
    rc, msg = _compiles(tmp_path, tmp_path, out.name, "int nb = LGB_EVR_NB_TUNED, b = LGB_TMA_BUDGET_TUNED;")
    assert rc == 0, msg


def test_factor_tuner_picks_the_fastest_cta_per_class(tmp_path, monkeypatch):
    def fake_time(nlat, npu, threads, repeat):
        return (1.0 if threads == 64 else 2.0), 100

    monkeypatch.setattr(tune_factor, "time_setup", fake_time)
    out = tmp_path / "lgb_factor_tune.h"
    monkeypatch.setattr(sys, "argv", ["tune_factor", "--out", str(out), "--repeat", "1"])
    assert tune_factor.main() == 0
    text = out.read_text()
    assert "lgb_factor_threads[LGB_NCLS] = {64, 64, 64, 64, 64, 64, 64, 64};" in text
    rc, msg = _compiles(tmp_path, tmp_path, out.name, "int first(void) { return lgb_factor_threads[0]; }")
    assert rc == 0, msg


def test_committed_tables_compile(tmp_path):
    for h, body in (("lgb_eval_tune.h", "int nb = LGB_EVR_NB_TUNED, b = LGB_TMA_BUDGET_TUNED;"),
                    ("lgb_factor_tune.h", "int first(void) { return lgb_factor_threads[0]; }")):
        rc, msg = _compiles(tmp_path, CSRC, h, body)
        assert rc == 0, msg
