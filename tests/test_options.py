"""Solver options in the reference's control.dat syntax (host only, no GPU):
the hot-path -ps_ksp_* options map onto cvb_solve_opts, comments and unrelated
options are skipped, later occurrences and command-line tokens override, and a
malformed value is a BAD_INPUT naming the option."""
import pytest


def test_control_file_and_overrides(tmp_path):
    from curvib_old_gb300 import _lib
    f = tmp_path / "control.dat"
    f.write_text("-ps_ksp_type fgmres\n"
                 "-ps_ksp_atol 1.e-5\n"
                 "-ps_ksp_rtol 1.e-11   # tolerance of the run\n"
                 "#-ps_ksp_gmres_restart 20\n"
                 "-ps_ksp_max_it 40\n"
                 "-mg_k_semi 1\n"
                 "-ps_ksp_monitor_true_residual\n"
                 "-cvb_precision fp64\n"
                 "-ps_ksp_max_it 60\n")
    o = _lib.opts_from_control(f)
    d = _lib.default_opts()
    assert (o.rtol, o.atol, o.max_it) == (1e-11, 1e-5, 60)
    assert o.restart == d.restart and o.precision == _lib.FP64
    o2 = _lib.opts_from_control(f, args=["-cvb_precision", "mixed", "-ps_ksp_gmres_restart", "20",
                                         "-cvb_smoother", "jacobi", "-cvb_omega", "0.9", "-cvb_pre_sweeps", "1"])
    assert o2.precision == _lib.MIXED and o2.restart == 20 and o2.smoother == _lib.JACOBI
    assert (o2.omega, o2.pre_sweeps, o2.rtol) == (0.9, 1, 1e-11)


@pytest.mark.parametrize("text", ["-ps_ksp_rtol abc\n", "-ps_ksp_max_it 4.5\n", "-cvb_precision fp16\n",
                                  "-ps_ksp_rtol\n"])
def test_malformed_values(tmp_path, text):
    from curvib_old_gb300 import _lib
    f = tmp_path / "control.dat"
    f.write_text(text)
    with pytest.raises(_lib.CvbError) as e:
        _lib.opts_from_control(f)
    assert e.value.status == _lib.CVB_BAD_INPUT and text.split()[0] in str(e.value)


def test_missing_file(tmp_path):
    from curvib_old_gb300 import _lib
    with pytest.raises(_lib.CvbError) as e:
        _lib.opts_from_control(tmp_path / "absent.dat")
    assert e.value.status == _lib.CVB_BAD_INPUT
