"""Generate the Sobol direction numbers used by the Sobol-Burley sample table.

The path-tracing pass reads a precomputed table of 4D Owen-scrambled Sobol
points (``sobol_burley::sample_4d(i, d, 0)`` for 17 dimension sets, reference
``src/pathtracing/pathtracer.rs:56-64``).  17 sets x 4 = 68 Sobol dimensions
are needed, with 32-bit direction numbers.

The primitive polynomials and initial direction numbers are the Joe & Kuo
(2008) ``new-joe-kuo-6.21201`` set as shipped with SciPy.  This script reads
that data, runs the Joe-Kuo recurrence to 32 bits, checks the result against
SciPy's own unscrambled Sobol generator (``bits=32``), and writes:

* ``nbounce_gb300/csrc/sobol_directions.inc`` - the 68 x 32 direction table
  compiled into the library;
* ``oracle/joe_kuo_68.inc`` - only the polynomials and initial values; the CPU
  oracle runs the recurrence itself, so the two sides are derived
  independently and both are pinned against SciPy by the tests.

Run from the repository root: ``python nbounce_gb300/csrc/gen_sobol_directions.py``.
"""
import os

import numpy as np

N_DIMS = 68
BITS = 32


def joe_kuo_data(n_dims=N_DIMS):
    import scipy.stats._sobol as s
    z = np.load(os.path.join(os.path.dirname(s.__file__), "_sobol_direction_numbers.npz"))
    return z["poly"][:n_dims].astype(np.int64), z["vinit"][:n_dims].astype(np.int64)


def direction_numbers(poly, vinit, bits=BITS):
    """V[dim][k] (k = 0 is the most significant bit) by the Joe-Kuo recurrence."""
    n = len(poly)
    V = np.zeros((n, bits), dtype=np.uint64)
    for k in range(bits):
        V[0, k] = 1 << (bits - 1 - k)
    for j in range(1, n):
        p = int(poly[j])
        s = p.bit_length() - 1               # polynomial degree
        a = (p >> 1) & ((1 << (s - 1)) - 1)  # inner coefficients a_1..a_{s-1}
        m = [0] * (bits + 1)                  # 1-based m_k
        for k in range(1, s + 1):
            m[k] = int(vinit[j][k - 1])
        for k in range(s + 1, bits + 1):
            v = m[k - s] ^ (m[k - s] << s)
            for i in range(1, s):
                if (a >> (s - 1 - i)) & 1:
                    v ^= m[k - i] << i
            m[k] = v
        for k in range(1, bits + 1):
            V[j, k - 1] = (m[k] << (bits - k)) & 0xFFFFFFFF
    return V.astype(np.uint32)


def sobol_points(V, n_points):
    """Unscrambled Sobol points in natural index order as uint32."""
    idx = np.arange(n_points, dtype=np.uint64)
    out = np.zeros((n_points, V.shape[0]), dtype=np.uint32)
    for k in range(V.shape[1]):
        bit = ((idx >> np.uint64(k)) & np.uint64(1)).astype(bool)
        out[bit] ^= V[:, k][None, :]
    return out


def check_against_scipy(V, n_points=1 << 12):
    from scipy.stats import qmc
    eng = qmc.Sobol(d=V.shape[0], scramble=False, bits=BITS)
    ref = (eng.random(n_points) * 2.0**32).astype(np.uint64).astype(np.uint32)
    ours = sobol_points(V, n_points)
    gray = np.arange(n_points) ^ (np.arange(n_points) >> 1)  # SciPy emits Gray-code order
    assert np.array_equal(ref, ours[gray]), "direction numbers disagree with SciPy"
    # the top direction numbers are only reached through index bits >= 12; pin them too
    for k in (20, 31):
        e = qmc.Sobol(d=V.shape[0], scramble=False, bits=BITS)
        p = (1 << (k + 1)) - 1          # Gray code of p is 1 << k
        e.fast_forward(p)
        got = (e.random(1)[0] * 2.0**32).astype(np.uint64).astype(np.uint32)
        assert np.array_equal(got, V[:, k]), f"direction bit {k} disagrees with SciPy"


def main():
    root = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    poly, vinit = joe_kuo_data()
    V = direction_numbers(poly, vinit)
    check_against_scipy(V)
    lines = ["// Generated by nbounce_gb300/csrc/gen_sobol_directions.py - do not edit.",
             f"// Sobol direction numbers (Joe & Kuo 2008), {N_DIMS} dimensions x {BITS} bits,",
             "// index [dim][k] with k = 0 the most significant bit.",
             f"static const unsigned int kSobolDirections[{N_DIMS}][{BITS}] = {{"]
    for j in range(N_DIMS):
        lines.append("  {" + ",".join(f"0x{int(x):08x}u" for x in V[j]) + "},")
    lines.append("};")
    with open(os.path.join(root, "nbounce_gb300", "csrc", "sobol_directions.inc"), "w") as f:
        f.write("\n".join(lines) + "\n")

    maxdeg = int(max(int(p).bit_length() - 1 for p in poly))
    lines = ["// Generated by nbounce_gb300/csrc/gen_sobol_directions.py - do not edit.",
             f"// Joe & Kuo (2008) primitive polynomials and initial direction numbers, first {N_DIMS} dimensions.",
             "// poly includes the leading and trailing coefficients; m holds m_1..m_s.",
             f"static const unsigned int kJoeKuoPoly[{N_DIMS}] = {{" + ",".join(str(int(p)) for p in poly) + "};",
             f"static const unsigned int kJoeKuoM[{N_DIMS}][{maxdeg}] = {{"]
    for j in range(N_DIMS):
        lines.append("  {" + ",".join(str(int(x)) for x in vinit[j][:maxdeg]) + "},")
    lines.append("};")
    with open(os.path.join(root, "oracle", "joe_kuo_68.inc"), "w") as f:
        f.write("\n".join(lines) + "\n")
    np.save(os.path.join(root, "tests", "golden", "sobol_unscrambled_68x256.npy"), sobol_points(V, 256))
    print("ok", V.shape)


if __name__ == "__main__":
    main()
