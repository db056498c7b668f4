"""The index algebra of in-place (AA pattern) streaming, on the CPU.

A numpy restatement of the two in-place steps (local: read A[q][x], write A[opp q][x]; stream: read
A[opp q][x - c_q], write A[q][x + c_q]) against the two-array pull step on a small periodic
lattice, with a stand-in collision that mixes a cell's populations (any per-cell map serves: the
identities are about where values live, not about BGK).  After t steps the in-place array must hold
A[q][x + c_q] = P_t[q][x] for even t and A[opp q][x] = P_t[q][x] for odd t; and every slot a step
writes is one it read (no value is overwritten before it is used)."""
import numpy as np

CX = [0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0]
CY = [0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1]
CZ = [0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1]
Q = 19


def opp(q):
    return 0 if q == 0 else (q + 1 if q & 1 else q - 1)


def shift(a, q, sign):
    """a moved by sign * c_q: result[x] = a[x - sign * c_q] (periodic); arrays are [z][y][x]."""
    return np.roll(a, (sign * CZ[q], sign * CY[q], sign * CX[q]), axis=(0, 1, 2))


def collide(f):
    """A per-cell stand-in for the collision: mixes all 19 populations of each cell, not symmetric in q."""
    s = f.sum(axis=0)
    return 0.7 * f + 0.3 * np.stack([np.sin(s + q) for q in range(Q)])


def pull_step(P):
    gathered = np.stack([shift(P[q], q, +1) for q in range(Q)])  # population q from x - c_q
    return collide(gathered)


def aa_step(A, t):
    A = A.copy()
    if t % 2 == 0:  # local: own slots in, population q out to slot opp(q)
        out = collide(A)
        for q in range(Q):
            A[opp(q)] = out[q]
    else:  # stream: population q from A[opp q] at x - c_q, out to A[q] at x + c_q
        gathered = np.stack([shift(A[opp(q)], q, +1) for q in range(Q)])
        out = collide(gathered)
        for q in range(Q):
            A[q] = shift(out[q], q, +1)
    return A


def aa_view(A, t):
    """P_t as the in-place array holds it after t steps."""
    if t % 2 == 0:
        return np.stack([shift(A[q], q, -1) for q in range(Q)])   # P[q][x] = A[q][x + c_q]
    return np.stack([A[opp(q)] for q in range(Q)])                # P[q][x] = A[opp q][x]


def test_inplace_layout_identities_hold_step_by_step():
    rng = np.random.default_rng(3)
    n = 5                                       # odd edge: every wrap-around is exercised
    P = rng.random((Q, n, n, n))
    A = np.stack([shift(P[q], q, +1) for q in range(Q)])   # the initial state written at x + c_q
    for t in range(7):
        np.testing.assert_allclose(aa_view(A, t), P, rtol=0, atol=0)
        P = pull_step(P)
        A = aa_step(A, t)


def test_each_inplace_step_writes_only_slots_it_read():
    # the stream step of the cell at x reads slots (opp q, x - c_q) and writes (q, x + c_q): over all
    # cells and q both are the same set, each slot once, so a thread owning those slots races no one
    n = 4
    cells = [(x, y, z) for z in range(n) for y in range(n) for x in range(n)]
    for x, y, z in cells:
        reads = {(opp(q), (x - CX[q]) % n, (y - CY[q]) % n, (z - CZ[q]) % n) for q in range(Q)}
        writes = {(q, (x + CX[q]) % n, (y + CY[q]) % n, (z + CZ[q]) % n) for q in range(Q)}
        assert reads == writes and len(reads) == Q
    all_reads = [(opp(q), (x - CX[q]) % n, (y - CY[q]) % n, (z - CZ[q]) % n) for x, y, z in cells for q in range(Q)]
    assert len(set(all_reads)) == Q * n ** 3          # every slot of the array read exactly once
