"""The LRU eviction walk's scan form against the one-entry-at-a-time walk.

k_evict_walk (csrc/k_map.cu) assigns victims to the creations of a batch that
overflow the capacity by a block-wide scan over the LRU queue instead of one
entry at a time.  This test restates both forms in Python and checks that
they give the same victims, the same final queue position, the same split
point and the same exhaustion on random queues, for scan widths from 1 to 64
entries (the kernel uses 1024).  The device kernel itself is checked against
the oracle by the eviction tests in test_gpu_parity.py.

Entry kinds: 0 stale (its voxel dead or touched again since), 1 live and not
touched in this batch, 2 live and first touched in this batch at tf.  The
creation j of the batch happens at point cg[j]; a touched entry whose first
touch precedes the creation it meets is skipped (it moved to the front), one
whose first touch follows it is the split point (the reference would evict
it and re-create it later in the batch).
"""
import random


def walk_serial(entries, j0, n_new, cg):
    q, victims = 0, []
    for j in range(j0, n_new):
        victim, split = None, None
        while q < len(entries):
            kind, tf, r = entries[q]
            q += 1
            if kind == 0:
                continue
            if kind == 2 and tf < cg[j]:
                continue
            victim = r
            if kind == 2:
                split = tf
            break
        if split is not None:
            return ("split", split)
        if victim is None:
            return ("exhausted", victims, q)
        victims.append(victim)
    return ("ok", victims, q)


def walk_scan(entries, j0, n_new, cg, width):
    need, q0, assigned, victims = n_new - j0, 0, 0, {}
    while True:
        step = entries[q0:q0 + width]
        rows, before = [], 0
        for t, (kind, tf, r) in enumerate(step):
            rows.append((t, kind, tf, r, assigned + before))  # the creation offset this entry meets
            before += kind == 1
        ts = min((t for t, kind, tf, r, a in rows if kind == 2 and a < need and tf >= cg[j0 + a]), default=width)
        last = -1
        for t, kind, tf, r, a in rows:
            if kind == 1 and t < ts and a < need:
                victims[a] = r
                if a == need - 1:
                    last = t
        if ts < width:
            return ("split", rows[ts][2])
        if last >= 0:
            return ("ok", [victims[i] for i in range(need)], q0 + last + 1)
        assigned += before
        q0 += width
        if q0 >= len(entries):
            return ("exhausted", [victims[i] for i in range(assigned)], len(entries))


def test_scan_walk_equals_serial_walk():
    rng = random.Random(1)
    checked = 0
    for _ in range(20000):
        n = rng.randint(0, 40)
        entries = [(rng.choice([0, 0, 1, 1, 1, 2]), rng.randint(0, 30), i) for i in range(n)]
        n_new = rng.randint(1, 12)
        j0 = rng.randint(0, n_new)
        if j0 >= n_new:
            continue
        cg = sorted(rng.sample(range(40), n_new))
        width = rng.choice([1, 3, 8, 64])
        assert walk_scan(entries, j0, n_new, cg, width) == walk_serial(entries, j0, n_new, cg)
        checked += 1
    assert checked > 15000
