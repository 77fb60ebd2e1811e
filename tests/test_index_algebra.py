"""Index algebra the sweep and observable kernels rely on, checked on the CPU.

The kernels replace per-amplitude work by per-part precomputation; each
replacement rests on an identity that is restated and checked here:
- successive tile bases by a masked add: deposit(v + g) equals deposit(v)
  plus deposit(g) with the carries passed through the tile bits;
- the shared-memory swizzle mixes only bits below 8, so the slot of element
  tid + 256 k is sw(tid) + 256 k, and it is GF(2)-linear;
- the CNOT-ladder map is GF(2)-linear, so an index's image is the XOR of
  its disjoint parts' images;
- the observable's diagonal: per-subset sums of the terms' signed weights
  and a Walsh-Hadamard transform over the element-loop bits give the same
  values as the per-amplitude term sum.
"""
import numpy as np
import pytest


def deposit(v, bits):
    x = 0
    for i, b in enumerate(bits):
        if (v >> i) & 1:
            x |= 1 << b
    return x


def sw128(e):
    return e ^ ((e >> 3) & 7)


def sw64(e):
    return e ^ ((e >> 4) & 15)


def ladder_masks(n):
    odd = even = 0
    for q in range(n - 1):
        b = 1 << (n - 1 - q)
        if q & 1:
            odd |= b
        else:
            even |= b
    return odd, even


def ladder_fwd(x, m):
    odd, even = m
    x ^= (x & odd) >> 1
    x ^= (x & even) >> 1
    return x


def ladder_inv(x, m):
    odd, even = m
    x ^= (x & even) >> 1
    x ^= (x & odd) >> 1
    return x


def tile_layouts(n, t, c):
    """Tile bit sets of the sweeps of a layer (sweep A, then high-bit sweeps
    that keep the c lowest bits), as the sweep program builds them."""
    tiles = [list(range(t))]
    nxt = t
    while nxt < n:
        k = min(t - c, n - nxt)
        tiles.append(list(range(t - k)) + list(range(nxt, nxt + k)))
        nxt += k
    return tiles


@pytest.mark.parametrize("n,t,c", [(24, 11, 3), (24, 12, 4), (20, 12, 4), (34, 13, 4), (17, 6, 3)])
def test_masked_add_tile_bases(n, t, c):
    rng = np.random.default_rng(n * 100 + t)
    for tile in tile_layouts(n, t, c):
        outside = [b for b in range(n) if b not in tile]
        tm = sum(1 << b for b in tile)
        omask = ((1 << n) - 1) & ~tm
        ntiles = 1 << len(outside)
        for grid in (1, 3, 152, 304, 456, int(rng.integers(2, 1000))):
            for start in {0, 1, min(grid - 1, ntiles - 1)}:
                nxt = deposit(start, outside)
                step = deposit(grid, outside)
                v = start
                for _ in range(40):
                    if v >= ntiles:
                        break
                    assert nxt == deposit(v, outside)
                    nxt = ((nxt | (~omask & ((1 << 64) - 1))) + step) & omask
                    v += grid


@pytest.mark.parametrize("sw", [sw128, sw64])
def test_swizzle_slot_split_and_linearity(sw):
    for tid in range(256):
        for k in range(32):
            assert sw(tid + 256 * k) == sw(tid) + 256 * k
    rng = np.random.default_rng(1)
    for _ in range(2000):
        a, b = (int(x) for x in rng.integers(0, 1 << 13, 2))
        assert sw(a ^ b) == sw(a) ^ sw(b)


@pytest.mark.parametrize("n", [2, 9, 24, 34])
def test_ladder_is_linear_and_inverse(n):
    m = ladder_masks(n)
    rng = np.random.default_rng(n)
    for _ in range(2000):
        a, b = (int(x) for x in rng.integers(0, 1 << n, 2, dtype=np.int64))
        assert ladder_fwd(a ^ b, m) == ladder_fwd(a, m) ^ ladder_fwd(b, m)
        assert ladder_inv(a ^ b, m) == ladder_inv(a, m) ^ ladder_inv(b, m)
        assert ladder_inv(ladder_fwd(a, m), m) == a


@pytest.mark.parametrize("n,t,seed", [(14, 12, 0), (16, 11, 1), (13, 10, 2), (12, 8, 3), (10, 7, 4)])
def test_observable_diagonal_by_subset_sums_and_transform(n, t, seed):
    """Element x = base | dep_lo(tid) | offhi(k) of tile A (bits 0..t-1): the
    kernel's D(k) for one thread and tile equals sum_j w_j (-1)^popc(x & m_j)."""
    rng = np.random.default_rng(seed)
    terms = []
    for q in range(n):
        if rng.random() < 0.5:
            terms.append((1 << q, float(rng.choice([0.5, -1.0, 0.25]))))
    for i in range(n):
        for j in range(i + 1, n):
            if rng.random() < 0.3:
                terms.append(((1 << i) | (1 << j), float(rng.choice([1.0, -0.5, 2.0]))))
    tile = list(range(t))
    kb = max(t - 8, 0)
    nk = 1 << kb
    kbits = tile[8:]
    outside = [b for b in range(n) if b not in tile]

    def subset(m):
        return sum(((m >> kbits[i]) & 1) << i for i in range(kb))

    for trial in range(12):
        tid = int(rng.integers(0, min(256, 1 << t)))
        tileid = int(rng.integers(0, 1 << (n - t)))
        bd = deposit(tileid, outside) | deposit(tid, tile[:8])
        b = np.zeros(16)
        for m, w in terms:
            b[subset(m)] += -w if bin(bd & m).count("1") & 1 else w
        for i in range(kb):  # butterflies over the element-loop bits
            for k in range(16):
                if not (k >> i) & 1 and (k | (1 << i)) < nk:
                    u, v = b[k], b[k | (1 << i)]
                    b[k], b[k | (1 << i)] = u + v, u - v
        for k in range(nk):
            x = bd | deposit(k << 8, tile) if t > 8 else bd
            direct = sum(-w if bin(x & m).count("1") & 1 else w for m, w in terms)
            assert b[k] == pytest.approx(direct, abs=1e-12)


# ---- batched kernel (qg_batched.cu, rotred_group)

def test_rescaled_reductions_after_unscaled_inverse_rotations():
    """The batched kernel's backward pass takes a rotation group's gradient
    sums after the earlier groups' unscaled inverse rotations (R(-theta) /
    kappa) have been applied to lambda and psi; the sums equal those at the
    layer's end point times 1/kappa^2 per such rotation.  Checked on a
    random 3-qubit state pair with numpy matrices."""
    rng = np.random.default_rng(9)
    X = np.array([[0, 1], [1, 0]], dtype=complex)
    Y = np.array([[0, -1j], [1j, 0]])
    I2 = np.eye(2)

    def on(op, q):  # qubit q of 3, q = 0 the most significant
        mats = [I2, I2, I2]
        mats[q] = op
        return np.kron(np.kron(mats[0], mats[1]), mats[2])

    lam = rng.normal(size=8) + 1j * rng.normal(size=8)
    psi = rng.normal(size=8) + 1j * rng.normal(size=8)
    th = rng.uniform(0, 2 * np.pi, 2)
    # rotation on qubit 0 (axis X) applied first, sum for qubit 1 (axis Y) after
    c, s = np.cos(th[0] / 2), np.sin(th[0] / 2)
    R_inv = c * I2 + 1j * s * X  # R_X(-theta)
    kappa = c if abs(c) >= abs(s) else s
    M = on(R_inv / kappa, 0)
    ref = np.imag(np.vdot(lam, on(Y, 1) @ psi))
    got = np.imag(np.vdot(M @ lam, on(Y, 1) @ (M @ psi)))
    assert abs(got * kappa ** 2 - ref) < 1e-12
