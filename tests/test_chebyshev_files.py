"""Output formats of the Chebyshev order-domain path (no GPU needed):
'chebyauto' (write_chebyshev_auto, chebyspec.f90:334-368, formats
'(a,2(2x,E21.14),/)' and '(i6,11x,E21.14)') and 'cheby1h1p' (write_1h1p
:372-394, unformatted sequential records)."""
import numpy as np

from adc_ottawa_gb300 import fortran_e, write_cheby1h1p, write_chebyshev_auto


def test_fortran_e_descriptor():
    assert fortran_e(1.0) == " 0.10000000000000E+01"
    assert fortran_e(-0.5) == "-0.50000000000000E+00"
    assert fortran_e(0.0) == " 0.00000000000000E+00"
    assert fortran_e(1.23456789012345678e-5) == " 0.12345678901235E-04"
    assert fortran_e(9.999999999999999) == " 0.10000000000000E+02"     # carry into the exponent
    assert fortran_e(1e120) == " 0.10000000000000+121"                # three-digit exponent drops the E
    assert all(len(fortran_e(x)) == 21 for x in (3.0, -2e-300, 7e99))


def test_chebyauto_layout(tmp_path):
    p = tmp_path / "chebyauto"
    write_chebyshev_auto(str(p), [-0.12, 25.5], [4.0, -1.5, 0.25])
    lines = p.read_text().split("\n")
    assert lines[0] == "#    Spectral bounds:  -0.12000000000000E+00   0.25500000000000E+02"
    assert lines[1] == ""
    assert lines[2] == "#    Order [k]    C_k"
    assert lines[3] == "     0            0.40000000000000E+01"
    assert lines[4] == "     1           -0.15000000000000E+01"
    assert len(lines[5]) == 6 + 11 + 21 and lines[6] == ""


def test_cheby1h1p_records(tmp_path):
    q = np.arange(12, dtype=np.float64).reshape(3, 4)     # 3 orders, n1 = 4
    p = tmp_path / "cheby1h1p"
    write_cheby1h1p(str(p), q)
    raw = p.read_bytes()
    assert len(raw) == 3 * (4 + 32 + 4)
    for k in range(3):
        rec = raw[k * 40:(k + 1) * 40]
        assert np.frombuffer(rec[:4], np.int32)[0] == 32 == np.frombuffer(rec[-4:], np.int32)[0]
        assert np.array_equal(np.frombuffer(rec[4:36], np.float64), q[k])
