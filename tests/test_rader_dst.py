"""The FP64 DST along R for npun2 = 256 (k_dst_rows_rader) on the CPU: the same
tables as the library's host set-up (3 a primitive root of 257, the Rader
kernel's FFT / 256, the output map), the same radix-4 Stockham passes and the
same read-off of y from W_j and W_{257-j}, against the DST-I product
y_i = sum_k 2 sin(pi i k / 257) x_k in long double."""
import numpy as np

N, M = 257, 256


def _tables():
    perm = [pow(3, q, N) for q in range(M)]
    col = [p - 1 for p in perm]
    out = []
    for p in range(M):
        j = perm[(M - p) % M]
        out.append((2 * j - 1, 0) if j <= 128 else (2 * j - 258, 1))
    tw = np.exp(-2j * np.pi * np.arange(M) / M)
    m = np.arange(M)
    d = np.exp(-2j * np.pi * np.array([perm[(M - k) % M] for k in m]) / N)
    ch = np.array([np.sum(d * np.exp(-2j * np.pi * ((m * k) % M) / M)) for k in range(M)]) / M
    return perm, col, out, tw, ch


def _stockham(x, tw):
    a, b = x.copy(), np.empty_like(x)
    ns = 1
    while ns < M:
        for t in range(M // 4):
            v = [a[t + 64 * r] for r in range(4)]
            if ns > 1:
                v = [v[r] * tw[(t % ns) * r * (64 // ns)] for r in range(4)]
            a0, a1, a2, a3 = v[0] + v[2], v[0] - v[2], v[1] + v[3], v[1] - v[3]
            d0 = (t // ns) * ns * 4 + t % ns
            b[d0], b[d0 + ns], b[d0 + 2 * ns], b[d0 + 3 * ns] = a0 + a2, a1 - 1j * a3, a0 - a2, a1 + 1j * a3
        a, b = b, a
        ns *= 4
    return a


def _dst_rader(x, tables):
    perm, col, out, tw, ch = tables
    a = np.array([x[c] * (1 + 1j * (1 if c & 1 else -1)) for c in col])
    r = _stockham(np.conj(_stockham(a, tw) * ch), tw)
    y = np.empty(M)
    for p in range(M):
        q = (p + 128) % M
        c, kind = out[p]
        y[c] = r[p].real - r[q].real if kind else r[p].imag - r[q].imag
    return y


def test_tables_cover_every_column():
    perm, col, out, tw, ch = _tables()
    assert sorted(perm) == list(range(1, N))
    assert sorted(c for c, _ in out) == list(range(M))
    assert pow(3, 128, N) == N - 1          # W_{257-j} sits 128 places from W_j


def test_stockham_is_the_dft():
    tw = _tables()[3]
    x = np.random.default_rng(0).standard_normal(M) + 1j * np.random.default_rng(1).standard_normal(M)
    assert np.allclose(_stockham(x, tw), np.fft.fft(x), rtol=0, atol=1e-12)


def test_rader_dst_matches_the_dense_product():
    tables = _tables()
    ld = np.longdouble
    i = np.arange(1, M + 1)
    arg = (np.outer(i, i) % (2 * N)).astype(ld)
    S = 2 * np.sin(ld(np.pi) * arg / ld(N))
    for seed in range(3):
        x = np.random.default_rng(seed).standard_normal(M)
        ref = S @ x.astype(ld)
        y = _dst_rader(x, tables)
        assert float(np.abs(y - ref).max() / np.abs(ref).max()) < 2e-15
