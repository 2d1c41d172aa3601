"""Seeded synthetic workloads for the vkhel hot path.

Prime rule: for degree n, scan downward from 2^60 over q = 1 (mod 2n) and
take the first prime (the first L distinct primes for L RNS limbs).  Root
rule: w = x^((q-1)/2n) for the smallest x >= 2 with w^n = -1 (mod q), i.e. a
primitive 2n-th root as the reference's negacyclic transform expects
(nt_is_primitive_root, src/numbers.c:61-69).  Operands are uniform in [0, q)
from numpy.random.default_rng(seed), drawn in the order instance -> limb ->
(a, b).
"""
import numpy as np

_MR_BASES = (2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37)


def is_prime(n):
    """Deterministic Miller-Rabin for n < 3.3e24 (covers all 64-bit n)."""
    if n < 2:
        return False
    for p in _MR_BASES:
        if n % p == 0:
            return n == p
    d, s = n - 1, 0
    while d % 2 == 0:
        d //= 2
        s += 1
    for a in _MR_BASES:
        x = pow(a, d, n)
        if x in (1, n - 1):
            continue
        for _ in range(s - 1):
            x = x * x % n
            if x == n - 1:
                break
        else:
            return False
    return True


def ntt_primes(n, count, bound=1 << 60):
    """First `count` primes q = 1 (mod 2n) below `bound`, scanning down."""
    out = []
    q = ((bound - 1) // (2 * n)) * (2 * n) + 1
    if q >= bound:
        q -= 2 * n
    while len(out) < count and q > 2 * n:
        if is_prime(q):
            out.append(q)
        q -= 2 * n
    return out


def root_for(n, q):
    """Smallest-x primitive 2n-th root w = x^((q-1)/2n) with w^n = -1."""
    e = (q - 1) // (2 * n)
    for x in range(2, 10000):
        w = pow(x, e, q)
        if pow(w, n, q) == q - 1:
            return w
    raise ValueError(f"no primitive 2n-th root found for n={n} q={q}")


def uniform(rng, q, size):
    return rng.integers(0, q, size=size, dtype=np.uint64)


def rns_batch(n, limbs, pairs, seed):
    """`pairs` RNS polynomial pairs of `limbs` limbs each: arrays (pairs, limbs, n)."""
    qs = ntt_primes(n, limbs)
    ws = [root_for(n, q) for q in qs]
    rng = np.random.default_rng(seed)
    a = np.empty((pairs, limbs, n), np.uint64)
    b = np.empty((pairs, limbs, n), np.uint64)
    for i in range(pairs):
        for k in range(limbs):
            a[i, k] = uniform(rng, qs[k], n)
            b[i, k] = uniform(rng, qs[k], n)
    return qs, ws, a, b


# The five configurations of the benchmark definition (degree, limbs, count).
CONFIGS = {
    "plain_small": dict(n=4096, limbs=1, pairs=1, seed=0),
    "single_limb_batch": dict(n=65536, limbs=1, pairs=64, seed=1),
    "rns_batch": dict(n=16384, limbs=8, pairs=32, seed=2),
}


def ragged_instances(count=512, seed=3, log_n_range=(12, 16), max_limbs=16):
    """Ragged batch: (log_n, limbs) per instance, log-uniform n, uniform limbs."""
    rng = np.random.default_rng(seed)
    log_ns = rng.integers(log_n_range[0], log_n_range[1] + 1, size=count)
    limbs = rng.integers(1, max_limbs + 1, size=count)
    return [(int(l), int(k)) for l, k in zip(log_ns, limbs)]


def ragged_batch(count=512, seed=3, log_n_range=(12, 16), max_limbs=16):
    """The ragged batch's operands: a list of (n, qs, ws, a, b), one per
    instance of ragged_instances(count, seed), with the instance's limbs
    taking the first `limbs` primes of its degree and a, b limb-major
    (limbs * n words); the operands come from default_rng(seed) drawn in
    instance order, all of a's limbs before b's."""
    rng = np.random.default_rng(seed)
    primes = {}
    out = []
    for log_n, limbs in ragged_instances(count, seed, log_n_range, max_limbs):
        n = 1 << log_n
        if n not in primes:
            qq = ntt_primes(n, max_limbs)
            primes[n] = (qq, [root_for(n, q) for q in qq])
        qs, ws = primes[n][0][:limbs], primes[n][1][:limbs]
        a = np.concatenate([uniform(rng, q, n) for q in qs])
        b = np.concatenate([uniform(rng, q, n) for q in qs])
        out.append((n, qs, ws, a, b))
    return out


def serving_requests(count, seed=4, log_n_range=(12, 17), max_limbs=24):
    """Polymul requests of the serving sweep: n = 2^k with k uniform in
    log_n_range, limbs uniform in 1..max_limbs (the first `limbs` primes of
    the degree), operands uniform mod each limb's prime, all from
    default_rng(seed): per request its shape, then a's limbs, then b's.
    Returns a list of (n, qs, ws, a, b), a and b limb-major."""
    rng = np.random.default_rng(seed)
    primes = {}
    out = []
    for _ in range(count):
        n = 1 << int(rng.integers(log_n_range[0], log_n_range[1] + 1))
        limbs = int(rng.integers(1, max_limbs + 1))
        if n not in primes:
            qq = ntt_primes(n, max_limbs)
            primes[n] = (qq, [root_for(n, q) for q in qq])
        qs, ws = primes[n][0][:limbs], primes[n][1][:limbs]
        a = np.concatenate([uniform(rng, q, n) for q in qs])
        b = np.concatenate([uniform(rng, q, n) for q in qs])
        out.append((n, qs, ws, a, b))
    return out
