"""Particle CSV input parsed on the device (csrc/csv.cu) against the host restatement.

The reference reads particle files line by line with std::stod / std::stoi
(runtime/read_from_file.hpp:33-116).  Here the bytes are indexed, parsed, filtered by
the domain test and compacted on the GPU.  Checked:
* every real field is the correctly rounded double of its decimal (bit-equal to
  Python's float) for the number formats particle files hold: the reference's own 6
  significant digits, shortest round-trip reprs (17 digits), fixed and exponent forms,
  signs, -0, white space, CRLF line ends, blank lines, a last line without a newline;
* the kept rows (domain test, infinite / fixed / global flags) equal the host's;
* a missing or malformed field and an int32 overflow fail with the line named, a
  number outside the exact range (more than 19 significant digits, or a decimal
  exponent beyond +-80) with a count;
* a user script's CSV input builds the same engine state as the host parse.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from pairs_gb300 import _capi as A  # noqa: E402
from pairs_gb300 import io  # noqa: E402

pytestmark = pytest.mark.gpu

REAL, INT = A.PG_CSV_REAL, A.PG_CSV_INT


def bits(x):
    return np.asarray(x, dtype=np.float64).view(np.int64)


def random_reals(rng, n):
    mag = 10.0 ** rng.uniform(-40, 40, n)
    x = rng.choice([-1.0, 1.0], n) * mag * rng.uniform(0.5, 1.0, n)
    # fixed notation only where it stays within 19 significant digits
    fmts = [repr, lambda v: "%.6g" % v, lambda v: "%.17e" % v, lambda v: ("%.12f" if abs(v) < 1e6 else "%.10e") % v,
            lambda v: "%.3e" % v, lambda v: "%+.9g" % v, lambda v: "  %.15g" % v, lambda v: "%.19g" % v]
    out = []
    for k, v in enumerate(x):
        out.append(fmts[k % len(fmts)](float(v)))
    out += ["0", "-0.0", "+0", "0.000", "1e0", "1E+2", "-2.5e-3", ".5", "5.", "007", "0.1", "123456789012345678",
            "9007199254740993", "9007199254740995", "1.5e27", "4.9e-27", "2.2250738585072014e-20", "1e-30",
            "8.5e-61", "1.2345678901234567e60", "0.30000000000000004", "2.5000000000000001e-05", "inf", "-NaN"]
    return out


def test_real_fields_are_correctly_rounded():
    rng = np.random.default_rng(11)
    fields = random_reals(rng, 20000)
    width = 4
    rows = [fields[i:i + width] for i in range(0, len(fields) - len(fields) % width, width)]
    text = "\n".join(",".join(r) for r in rows) + "\n"
    tab = io.csv_table_device(text.encode(), [REAL] * width).cpu().numpy()
    want = np.array([[float(v) for v in r] for r in rows]).T
    assert tab.shape == want.shape
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(tab), nan)
    assert np.array_equal(bits(tab[~nan]), bits(want[~nan]))


def test_layout_blank_lines_crlf_and_integers():
    text = ("1, 0, 4, 1.5, 0.25, 0.5, 0.75\r\n"
            "\n"
            "   \n"
            "2,1,0,2.0,1e-3,-0.0,3.5\r\n"
            "3,+2,-7,  2.5 ,1,2,3")                   # last line without a newline
    kinds = [INT, INT, INT, REAL, REAL, REAL, REAL]
    tab = io.csv_table_device(text.encode(), kinds).cpu().numpy()
    want = np.array([[1, 0, 4, 1.5, 0.25, 0.5, 0.75], [2, 1, 0, 2.0, 1e-3, -0.0, 3.5],
                     [3, 2, -7, 2.5, 1, 2, 3]], dtype=np.float64).T
    assert np.array_equal(bits(tab), bits(want))
    assert io.csv_table_device(b"", kinds).shape == (7, 0)


def test_domain_filter_and_flags_match_the_host():
    rng = np.random.default_rng(5)
    n = 5000
    pos = rng.uniform(-1.0, 11.0, (n, 3))
    pos[:50, 0] = 10.0 - 1e-5                          # on the reference's upper edge: dropped
    pos[50:100, 1] = 0.0                               # on the lower edge: kept
    flags = rng.choice([0, 0, 0, 1, 2, 4, 8], n)
    lines = ["%d,%d,%r,%r,%r,1.0" % (i, int(flags[i]), *pos[i].tolist()) for i in range(n)]
    text = "\n".join(lines) + "\n"
    kinds = [INT, INT, REAL, REAL, REAL, REAL]
    lo, hi = [0.0] * 3, [10.0] * 3
    tab = io.csv_table_device(text.encode(), kinds, pos_field=2, flags_field=1, lo=lo, hi=hi).cpu().numpy()
    inside = np.all((pos >= 0.0) & (pos < np.float64(10.0) - 0.00001), axis=1)
    keep = inside | ((flags & 13) != 0)
    assert tab.shape[1] == int(keep.sum())
    assert np.array_equal(tab[0].astype(np.int64), np.arange(n)[keep])      # file order
    assert np.array_equal(bits(tab[2:5].T), bits(pos[keep]))


@pytest.mark.parametrize("text,line", [("1,2,3\n4,5\n", 2), ("1,2,3\n4,x,6\n", 2), ("1,2,\n", 1),
                                       ("1,2,3\n1,2,3\n3000000000,1,1\n", 3)])
def test_malformed_lines_are_named(text, line):
    with pytest.raises(A.PairsError, match=f"line {line} "):
        io.csv_table_device(text.encode(), [INT, REAL, REAL])


def test_numbers_outside_the_exact_range_fail():
    for v in ("1e-90", "1.2345678901234567e99", "1.00000000000000000001"):
        with pytest.raises(A.PairsError, match="exact conversion"):
            io.csv_table_device(("1,%s\n" % v).encode(), [INT, REAL])
    # trailing zeros beyond 19 digits and a prefix read as std::stod reads it are fine
    tab = io.csv_table_device(b"1,1.00000000000000000000000,2.5abc\n", [INT, REAL, REAL]).cpu().numpy()
    assert tab[1, 0] == 1.0 and tab[2, 0] == 2.5


def test_user_script_input_matches_the_host_parse(tmp_path):
    import pairs_gb300 as pairs
    from tests.scripts import md_script
    rng = np.random.default_rng(3)
    n = 2000
    L = 4 * 1.6796
    pos = rng.uniform(-0.5, L + 0.5, (n, 3))
    rows = ["%d,0,%d,1.0,%r,%r,%r,%.6g,%.6g,%.6g" % (i, 4 if i % 97 == 0 else 0, *pos[i].tolist(),
                                                    *rng.normal(size=3).tolist())
            for i in range(n)]
    f = tmp_path / "p.input"
    f.write_text("\n".join(rows) + "\n")
    psim = md_script.build(pairs, nx=4, input_file=str(f))
    names = ['uid', 'type', 'flags', 'mass', 'position', 'linear_velocity']
    dev = io.read_particle_data(psim, str(f), names, pairs.point_mass(), device=True)
    host = io.read_particle_data(psim, str(f), names, pairs.point_mass(), device=False)
    assert set(dev) == set(host)
    for k in host:
        assert np.array_equal(np.asarray(dev[k]), np.asarray(host[k])), k
    assert 0 < len(dev["uid"]) < n
