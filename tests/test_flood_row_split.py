"""The flood's row update on a lane pair (relax_half in csrc/vf_flood.cu):
each half of a 32-voxel row runs its forward and backward in-row chain from a
lower bound of the chain value at the half boundary, then takes the exact
boundary value from the other half and raises its keys while step^d(P) exceeds
them.  This model of that scheme must equal the sequential row pass for any
row, halo keys and cross-row candidates (the chain is max-plus linear along an
occupied run).  Host-side check of the algebra; the GPU tests check the kernel
against the oracle."""
import random

S = 4096  # one BFS step in key units


def step(m):
    return m - S if m >= 2 * S else 0


def relax(kk, m):
    return max(kk, step(m)) if kk else 0


def chain(a, occ, prev):
    return max(a, prev - S if (occ and prev >= 2 * S) else 0)


def sequential(kk, w, hlo, hhi):
    f = list(kk)
    prev = hlo
    for z in range(32):
        f[z] = chain(relax(kk[z], w[z]), kk[z] != 0, prev)
        prev = f[z]
    prev = hhi
    for z in range(31, -1, -1):
        f[z] = chain(f[z], f[z] != 0, prev)
        prev = f[z]
    return f


def fix_up(f, P, zs):
    v = P
    for z in zs:
        v = v - S if (f[z] != 0 and v >= 2 * S) else 0
        if v <= f[z]:
            break
        f[z] = v


def lane_pair(kk, w, hlo, hhi, lower_bound):
    f = list(kk)
    # forward: lane 0 exact from hlo, lane 1 from a lower bound of f[15]
    prev = hlo
    for z in range(16):
        f[z] = chain(relax(kk[z], w[z]), kk[z] != 0, prev)
        prev = f[z]
    P = prev
    prev = lower_bound(kk[15], f[15])
    for z in range(16, 32):
        f[z] = chain(relax(kk[z], w[z]), kk[z] != 0, prev)
        prev = f[z]
    fix_up(f, P, range(16, 32))
    # backward: lane 1 exact from hhi, lane 0 from a lower bound of f[16]
    prev = hhi
    for z in range(31, 15, -1):
        f[z] = chain(f[z], f[z] != 0, prev)
        prev = f[z]
    P2 = f[16]
    prev = lower_bound(kk[16], f[16])
    for z in range(15, -1, -1):
        f[z] = chain(f[z], f[z] != 0, prev)
        prev = f[z]
    fix_up(f, P2, range(15, -1, -1))
    return f


def test_lane_pair_row_update_equals_sequential_pass():
    rng = random.Random(2024)
    for trial in range(20000):
        base = rng.randint(40, 400)
        occupied = rng.choice([0.5, 0.8, 0.95, 1.0])

        def key():
            if rng.random() < 0.3:
                return 1  # occupied, not reached
            return (1 << 31) - ((base + rng.randint(-20, 20)) * S + rng.randint(0, 50))

        kk = [key() if rng.random() < occupied else 0 for _ in range(32)]
        w = [key() if rng.random() < 0.5 else 0 for _ in range(32)]
        hlo = key() if rng.random() < 0.7 else 0
        hhi = key() if rng.random() < 0.7 else 0
        # the boundary value a lane reads may be the key before or after the
        # other lane's update: either is a lower bound of the exact value
        pick = (lambda old, new: old) if trial % 2 else (lambda old, new: new)
        assert lane_pair(kk, w, hlo, hhi, pick) == sequential(kk, w, hlo, hhi), trial
