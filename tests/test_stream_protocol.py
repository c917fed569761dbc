"""CPU model of the streamed host-buffer trace's copy-out protocol (csrc/trace_stream.cuh: claim_leader, late_held,
jump_done, finalize_done; the per-warp refill loop of csrc/trace_bvh4.cu and trace_persistent.cu).

Warps of 32 lanes take rays from one counter in batches once enough lanes are idle; rays run for random numbers of
steps (a heavy tail of long rays); a finished ray's hit is written at the warp's next refill.  Each warp counts the
rays it claims in two open parts, publishes the older one when its claims move two parts on, and late-lists the
rays it still holds in a part it publishes; at exhaustion it publishes both and late-lists everything it holds.

Checked for many seeds, part sizes, warp counts and refill thresholds:
  * every part's counter ends exactly at its size and never exceeds it (the copy-out waits end, and never early);
  * every ray is counted exactly once and late-listed at most once (the late list fits in ray_count entries);
  * every ray's host record is final: its hit was written before its part's counter completed (the part copy
    takes it), or it is late-listed (the late scatter, after every part copy, writes it).
"""
import random

import pytest

INVALID = 0xFFFFFFFF


def simulate(seed, count, pshift, warps, refill_min, tail, arrive_miss):
    rnd = random.Random(seed)
    nparts = (count + (1 << pshift) - 1) >> pshift
    size = [min(1 << pshift, count - (p << pshift)) for p in range(nparts)]
    done = [0] * nparts
    complete_t = [None] * nparts
    counted = [0] * count
    written_t = [None] * count
    late = []
    ctr = 0
    clock = 0

    def part(g):
        return g >> pshift

    def publish(p, v):
        done[p] += v
        assert done[p] <= size[p], "a part's counter passed its size"
        if done[p] == size[p]:
            complete_t[p] = clock

    class Warp:
        def __init__(self):
            self.active = [False] * 32
            self.pending = [False] * 32
            self.gid = [None] * 32
            self.left = [0] * 32
            self.exhausted = False
            self.cur_c, self.cur_n, self.prev_c, self.prev_n, self.fin = 0, 0, INVALID, 0, False

        def held(self, lane):
            return self.active[lane] or self.pending[lane]

    def duration():
        return rnd.randint(1, 20) if rnd.random() > tail else rnd.randint(50, 3000)

    def claim(w, base, end):
        # claim_leader, then late_held by every lane
        hi, lo = (end - 1) >> pshift, base >> pshift
        assert hi <= lo + 1, "a claim spans at most two parts"
        cur_c = w.cur_c
        if hi > cur_c:
            if w.prev_n:
                publish(w.prev_c, w.prev_n)
            late_part = w.prev_c
            w.prev_c, w.prev_n, w.cur_c, w.cur_n = cur_c, w.cur_n, hi, 0
            for lane in range(32):
                if w.held(lane) and part(w.gid[lane]) == late_part:
                    late.append(w.gid[lane])
        hs = hi << pshift
        in_prev = base < hs and lo == cur_c
        w.cur_n += end - max(base, hs)
        if in_prev:
            w.prev_n += hs - base
        for g in range(base, end):
            counted[g] += 1
        return hs if base < hs and not in_prev else 0

    def jump(w, fresh, jump_end):
        k = 0
        for lane in range(32):
            if fresh[lane] and w.gid[lane] < jump_end:
                late.append(w.gid[lane])
                k += 1
        if k:
            publish(part(jump_end - 1), k)

    def finalize(w):
        if w.fin:
            return
        for lane in range(32):
            if w.held(lane) and part(w.gid[lane]) in (w.cur_c, w.prev_c):
                late.append(w.gid[lane])
        if w.cur_n:
            publish(w.cur_c, w.cur_n)
        if w.prev_n:
            publish(w.prev_c, w.prev_n)
        w.cur_n = w.prev_n = 0
        w.fin = True

    ws = [Warp() for _ in range(warps)]
    live = list(range(warps))
    while live:
        wi = rnd.choice(live)
        w = ws[wi]
        clock += 1
        nidle = sum(not a for a in w.active)
        if nidle and (nidle >= refill_min or w.exhausted or nidle == 32):
            n = 0 if w.exhausted else nidle
            base, jump_end = 0, 0
            if n:
                base, ctr = ctr, ctr + n
                w.exhausted = base + n >= count
                if base < count:
                    jump_end = claim(w, base, min(base + n, count))
            fresh = [False] * 32
            k = 0
            for lane in range(32):
                if w.active[lane]:
                    continue
                if w.pending[lane]:
                    written_t[w.gid[lane]] = clock
                    w.pending[lane] = False
                my = base + k
                k += 1
                if n and my < count:
                    w.gid[lane] = my
                    fresh[lane] = True
                    if rnd.random() < arrive_miss:  # a chunk that never arrived: a miss at the next refill
                        w.pending[lane] = True
                    else:
                        w.active[lane] = True
                        w.left[lane] = duration()
            if jump_end:
                jump(w, fresh, jump_end)
            if w.exhausted:
                finalize(w)
        if not any(w.active) and w.exhausted and not any(w.pending):
            assert w.fin and w.cur_n == 0 and w.prev_n == 0
            live.remove(wi)
            continue
        for lane in range(32):
            if w.active[lane]:
                w.left[lane] -= 1
                if w.left[lane] <= 0:
                    w.active[lane] = False
                    w.pending[lane] = True
    assert done == size, "every part's counter reaches its size"
    assert all(c == 1 for c in counted), "every ray counted once"
    assert len(late) == len(set(late)) <= count, "late-listed at most once"
    listed = set(late)
    stale = [g for g in range(count) if g not in listed and written_t[g] > complete_t[part(g)]]
    assert not stale, f"rays whose host record would be stale: {stale[:5]}"
    return len(late)


@pytest.mark.parametrize("seed", range(24))
def test_copy_out_protocol(seed):
    rnd = random.Random(seed)
    count = rnd.choice([1, 31, 33, 1000, 4096, 5000, 12289])
    pshift = rnd.choice([5, 6, 8, 10])
    warps = rnd.choice([1, 3, 16, 48])
    simulate(seed, count, pshift, warps, refill_min=rnd.choice([1, 8, 32]), tail=rnd.choice([0, 0.01, 0.2]),
             arrive_miss=rnd.choice([0, 0.01]))


def test_long_rays_are_late_listed():
    """With a heavy tail of long rays and small parts, parts are published while rays are in flight."""
    assert simulate(7, 12289, 6, 16, refill_min=8, tail=0.2, arrive_miss=0) > 0
