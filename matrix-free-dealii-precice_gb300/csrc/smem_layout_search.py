"""Search of the padded shared-memory layouts of cell_apply_kernel
(ApplyPad in mf_cell.cuh): row stride SY, plane stride SZ and cell stride SC
(elements) that minimise the shared-memory wavefronts of the line sweeps.

Model: thread t of a block belongs to cell t / N^2 and owns line (a, b) with
a = l % N, b = l / N (l = t % N^2); in sweep direction d every thread
accesses element i of its line at the same time.  4-byte elements: one
phase of 32 threads over 32 banks; 8-byte elements: two half-warp phases,
each element on two banks.  Wavefronts of an access = the largest number of
distinct words on one bank, summed over phases.  Run with no arguments to
print the table (4-byte padding up to 25 %, 8-byte up to 2 %)."""
import itertools, sys

CPB = {(2, 4): 32, (3, 4): 32, (4, 4): 8, (5, 4): 5, (6, 4): 7, (7, 4): 5,
       (2, 8): 32, (3, 8): 32, (4, 8): 8, (5, 8): 5, (6, 8): 5, (7, 8): 3}
NARR = 12  # arrays per cell (NC * 4)

def wavefronts(addrs, es):
    """addrs: element offsets accessed by the 32 threads (None = inactive)."""
    if es == 4:
        phases = [addrs]
    else:
        phases = [addrs[:16], addrs[16:]]
    total = 0
    for ph in phases:
        banks = {}
        for a in ph:
            if a is None:
                continue
            for w in ([a] if es == 4 else [2 * a, 2 * a + 1]):
                banks.setdefault(w % 32, set()).add(w if es == 4 else a)
        total += max((len(v) for v in banks.values()), default=0)
    return total

def cost(N, es, SY, SZ, SC):
    cpb = CPB[(N, es)]
    nthr = cpb * N * N
    tot = 0
    for w0 in range(0, nthr, 32):
        for d in range(3):
            for i in range(N):
                addrs = []
                for t in range(w0, w0 + 32):
                    if t >= nthr:
                        addrs.append(None); continue
                    c, l = divmod(t, N * N)
                    a, b = l % N, l // N
                    if d == 0:   base, st = a * SY + b * SZ, 1
                    elif d == 1: base, st = a + b * SZ, SY
                    else:        base, st = a + b * SY, SZ
                    addrs.append(c * SC + base + i * st)
                tot += wavefronts(addrs, es)
    return tot

for es in (4, 8):
    for N in range(2, 8):
        nat = cost(N, es, N, N * N, NARR * N ** 3)
        best = None
        for SY in range(N, N + 5):
            for SZ in range(N * SY, N * SY + 9):
                base_cell = NARR * SZ * N
                for SC in range(base_cell, base_cell + 33):
                    over = SC / (NARR * N ** 3) - 1
                    if over > (0.25 if es == 4 else 0.02):
                        continue
                    c = cost(N, es, SY, SZ, SC)
                    key = (c, over)
                    if best is None or key < best[0]:
                        best = (key, SY, SZ, SC)
        (c, over), SY, SZ, SC = best
        print(f"es={es} N={N}: natural {nat} -> {c} wavefronts ({c/nat:.2f}x), SY={SY} SZ={SZ} SC={SC} (+{100*over:.1f}% smem)", flush=True)
