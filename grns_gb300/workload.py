"""Seeded synthetic workloads (numpy), identical on every machine.

Counter-based generator: every value is a pure function of (seed, stream,
counter), so any element of any array can be regenerated independently.

    splitmix64(z) = finaliser of z + 0x9E3779B97F4A7C15 (Steele, Lea, Flood 2014)
    draw(seed, stream, ctr) = splitmix64(splitmix64(seed ^ (stream << 32)) + ctr)

* uniform X in [0, M): independent uniform residues per modulus (exact by
  CRT), each by Lemire's multiply-shift with rejection (up to 4 attempts,
  counter = (k * n + i) * 4 + attempt);
* divisor of bit length L, L uniform in [1, log2M]: 32-bit limbs, top limb
  masked to L bits with its top bit set, reduced per modulus by Horner;
* power-of-two exponents D uniform in [1, Dmax];
* mp_int magnitudes uniform in [0, 2^bits) as 32-bit limbs, sign a fair coin
  (zero has sign 0).
The same definitions are used by the device generator (csrc/gen.cu).
"""
import numpy as np

MASK64 = (1 << 64) - 1
GOLDEN = 0x9E3779B97F4A7C15

# streams
S_X, S_Y, S_DLEN, S_DLIMB, S_SHIFT, S_MAG, S_SIGN, S_MAX = 1, 2, 3, 4, 5, 6, 7, 8


def _splitmix(z):
    """vectorised splitmix64 on uint64 arrays (wrapping arithmetic)"""
    with np.errstate(over="ignore"):
        z = z + np.uint64(GOLDEN)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def draw(seed, stream, ctr):
    key = _splitmix(np.uint64((seed ^ (stream << 32)) & MASK64))
    with np.errstate(over="ignore"):
        return _splitmix(key + np.asarray(ctr, dtype=np.uint64))


def _mulhi_lo(u, m):
    """128-bit product u * m (u uint64 array, m < 2^32): (high64, low64)"""
    m = np.uint64(m)
    lo32 = u & np.uint64(0xFFFFFFFF)
    hi32 = u >> np.uint64(32)
    with np.errstate(over="ignore"):
        a = lo32 * m
        b = hi32 * m
        high = (b + (a >> np.uint64(32))) >> np.uint64(32)
        low = (b << np.uint64(32)) + a
    return high, low


def uniform_residues(moduli, count, seed, stream, layout="soa"):
    """int32 residues of `count` numbers uniform in [0, M)."""
    n = len(moduli)
    out = np.empty((n, count), dtype=np.int32)
    k = np.arange(count, dtype=np.uint64)
    for i, m in enumerate(moduli):
        thr = np.uint64(((1 << 64) - m) % m)
        res = np.zeros(count, dtype=np.uint64)
        todo = np.ones(count, dtype=bool)
        for a in range(4):
            u = draw(seed, stream, (k * np.uint64(n) + np.uint64(i)) * np.uint64(4) + np.uint64(a))
            hi, lo = _mulhi_lo(u, m)
            ok = todo & (lo >= thr)
            res[ok] = hi[ok]
            if a == 3:
                res[todo & ~ok] = hi[todo & ~ok]
            todo &= ~ok
            if not todo.any():
                break
        out[i] = res.astype(np.int32)
    return out if layout == "soa" else np.ascontiguousarray(out.T)


def bit_lengths(log2M, count, seed, stream=S_DLEN):
    """L uniform in [1, log2M]"""
    u = draw(seed, stream, np.arange(count, dtype=np.uint64))
    hi, _ = _mulhi_lo(u, log2M)
    return (hi + np.uint64(1)).astype(np.int64)


def random_limbs(bits_per_elem, count, seed, stream, top_bit=True):
    """Python ints: element k has exactly bits_per_elem[k] bits (top bit set when top_bit)."""
    out = []
    for k in range(count):
        L = int(bits_per_elem[k])
        nl = (L + 31) // 32
        w = draw(seed, stream, np.arange(nl, dtype=np.uint64) + np.uint64(k) * np.uint64(64))
        v = 0
        for j in range(nl):
            v |= (int(w[j]) & 0xFFFFFFFF) << (32 * j)
        v &= (1 << L) - 1
        if top_bit:
            v |= 1 << (L - 1)
        out.append(v)
    return out


def divisors(moduli, log2M, count, seed, layout="soa"):
    """divisor residues (bit length uniform in [1, log2M]) and the Python ints"""
    L = bit_lengths(log2M, count, seed)
    vals = random_limbs(L, count, seed, S_DLIMB, top_bit=True)
    return to_residues(vals, moduli, layout), vals


def shifts(count, dmax, seed, stream=S_SHIFT):
    """D uniform in [1, dmax] (uint32)"""
    u = draw(seed, stream, np.arange(count, dtype=np.uint64))
    hi, _ = _mulhi_lo(u, dmax)
    return (hi + np.uint64(1)).astype(np.uint32)


def to_residues(values, moduli, layout="soa"):
    arr = np.array([[v % m for v in values] for m in moduli], dtype=np.int64).astype(np.int32)
    arr = arr.reshape(len(moduli), len(values))
    return arr if layout == "soa" else np.ascontiguousarray(arr.T)


def from_residues(res, moduli, layout="soa"):
    """Python ints from residues by CRT"""
    res = np.asarray(res)
    if layout != "soa":
        res = res.T
    M = 1
    for m in moduli:
        M *= m
    basis = [(M // m) * pow(M // m, -1, m) for m in moduli]
    cols = res.shape[1]
    return [sum(int(res[i, k]) * basis[i] for i in range(len(moduli))) % M for k in range(cols)]


def mpint_values(count, bits, seed):
    """signed Python ints: magnitude uniform in [0, 2^bits), fair-coin sign, zero has sign 0"""
    mags = random_limbs(np.full(count, bits), count, seed, S_MAG, top_bit=False)
    s = draw(seed, S_SIGN, np.arange(count, dtype=np.uint64)) & np.uint64(1)
    return [(-v if (int(b) and v) else v) for v, b in zip(mags, s)]
