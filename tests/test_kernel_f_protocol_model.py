"""CPU model check of the synchronisation protocol of the fused LCA timestep kernel
(step_tc_kernel, openpv_gb300/csrc/lca_solver.cu).

Every role of one CTA runs as a coroutine over exact mbarrier semantics (a wait on parity p passes
once the barrier has completed a phase of the other parity; a barrier completes a phase when its
expected arrivals are in), and a random scheduler interleaves them with the completions of
asynchronous copies (TMA / bulk loads, in any order) and of tcgen05 commits (in issue order).
The roles and hand-offs follow the kernel:

  weight loader   per block: wEmpty[slot] (previous use) -> wFull[slot] (TMA)
  V/stage loader  event loop: the next tile's stage once stEmpty(t-1) and foldFree(t-2); the next
                  block's V chunk once vEmpty[slot] (previous use)
  MMA             event loop: GEMM1 of block g1 needs imFull (a tile's first block), wFull[slot],
                  accEmpty[g1 % 2] (g1 >= 2) -> commits accFull, imEmpty (a tile's last block);
                  GEMM2 of block g2 < g1 needs aFull[g2 % 2] and, at a tile's first block, d2Empty
                  of the previous tile -> commits aEmpty, wEmpty, d2Full (a tile's last block)
  epilogue        two groups of 8 warps on alternating blocks: release a pending V slot, wait
                  accFull and vFull, arrive accEmpty, wait aEmpty (previous A tile of the group),
                  arrive aFull, store V; the V slot goes back at once with 2 slots, at the top of
                  the group's next block with 4
  tile warps      4 warps on one named barrier: im2col(0), then per tile im2col(t+1), fold(t);
                  im2col: stFull, barrier, imEmpty(t-1), barrier, barrier -> imFull, stEmpty;
                  fold: barrier, x load + d2Full, barrier, 16 tap-group barriers with d2Empty
                  after the last TMEM load (before the last 4), barrier -> foldFree

A run passes when every role finishes, every barrier ends on a phase boundary and no wait ever
observed a barrier more than one phase away from the one it waits for (parity aliasing).
"""
import random

import pytest


class _Barrier:
    def __init__(self, count, clock):
        self.count, self.pending, self.done, self.clock = count, 0, 0, clock

    def arrive(self):
        self.clock[0] += 1
        self.pending += 1
        assert self.pending <= self.count, "more arrivals than the barrier expects"
        if self.pending == self.count:
            self.pending = 0
            self.done += 1


def run_protocol(n_blk, n_v, n_w, tiles, seed, max_steps=2_000_000):
    """Returns 'ok', or a description of the deadlock or hazard found."""
    rnd = random.Random(seed)
    clock = [0]
    hazards = []
    q_total = tiles * n_blk
    bars = {}

    def mk(name, count=1):
        bars[name] = _Barrier(count, clock)

    for n in ("stFull", "stEmpty", "imFull", "imEmpty", "d2Full", "foldFree", "xFull"):
        mk(n)
    mk("d2Empty", 4)
    for i in range(n_w):
        mk(f"wFull{i}")
        mk(f"wEmpty{i}")
    for i in range(n_v):
        mk(f"vFull{i}")
        mk(f"vEmpty{i}", 8)
    for i in range(2):
        mk(f"accFull{i}")
        mk(f"accEmpty{i}", 8)
        mk(f"aFull{i}", 8)
        mk(f"aEmpty{i}")
    async_q, commit_q = [], []
    named = {}

    def test(name, k):
        """Phase k of the barrier completed (the kernel's parity test, k & 1)."""
        d = bars[name].done
        if d < k or d > k + 1:
            hazards.append((name, k, d))
        return (d & 1) != (k & 1)

    def wait(name, k):
        while not test(name, k):
            yield "blocked"

    def barsync(n):
        st = named.setdefault(1, [0, 0])
        gen = st[1]
        st[0] += 1
        clock[0] += 1
        if st[0] == n:
            st[0] = 0
            st[1] += 1
        while named[1][1] == gen:
            yield "blocked"

    def weight_loader():
        sw = uw = 0
        for _ in range(q_total):
            if uw > 0:
                yield from wait(f"wEmpty{sw}", uw - 1)
            async_q.append(f"wFull{sw}")
            yield "step"
            sw += 1
            if sw == n_w:
                sw, uw = 0, uw + 1

    def v_stage_loader():
        st_next = vq = sv = uv = 0
        while st_next < tiles or vq < q_total:
            did = False
            if st_next < tiles and (st_next == 0 or test("stEmpty", st_next - 1)) and \
                    (st_next < 2 or test("foldFree", st_next - 2)):
                async_q.append("stFull")
                st_next += 1
                did = True
            if vq < q_total and (uv == 0 or test(f"vEmpty{sv}", uv - 1)):
                async_q.append(f"vFull{sv}")
                vq += 1
                did = True
                sv += 1
                if sv == n_v:
                    sv, uv = 0, uv + 1
            yield "step" if did else "blocked"

    def mma():
        g1 = ti1 = nb1 = sw1 = uw1 = 0
        g2 = nb2 = sw2 = ti2 = 0
        while g2 < q_total:
            did = False
            if g1 < q_total:
                a = g1 & 1
                if (nb1 != 0 or test("imFull", ti1)) and test(f"wFull{sw1}", uw1) and \
                        (g1 < 2 or test(f"accEmpty{a}", g1 // 2 - 1)):
                    commit_q.append(f"accFull{a}")
                    if nb1 == n_blk - 1:
                        commit_q.append("imEmpty")
                    g1 += 1
                    sw1 += 1
                    if sw1 == n_w:
                        sw1, uw1 = 0, uw1 + 1
                    nb1 += 1
                    if nb1 == n_blk:
                        nb1, ti1 = 0, ti1 + 1
                    did = True
            if g2 < g1 and test(f"aFull{g2 & 1}", g2 >> 1) and (nb2 != 0 or ti2 == 0 or test("d2Empty", ti2 - 1)):
                commit_q.append(f"aEmpty{g2 & 1}")
                commit_q.append(f"wEmpty{sw2}")
                if nb2 == n_blk - 1:
                    commit_q.append("d2Full")
                g2 += 1
                sw2 = (sw2 + 1) % n_w
                nb2 += 1
                if nb2 == n_blk:
                    nb2, ti2 = 0, ti2 + 1
                did = True
            yield "step" if did else "blocked"

    def epilogue(warp):
        g = warp >> 3
        pending = -1
        for q in range(g, q_total, 2):
            sv, uv, k = q % n_v, q // n_v, q >> 1
            if pending >= 0:
                bars[f"vEmpty{pending}"].arrive()
                pending = -1
            yield from wait(f"accFull{g}", k)
            yield from wait(f"vFull{sv}", uv)
            bars[f"accEmpty{g}"].arrive()
            yield "step"  # the update
            if k >= 1:
                yield from wait(f"aEmpty{g}", k - 1)
            bars[f"aFull{g}"].arrive()
            yield "step"  # the V store
            if n_v == 2:
                bars[f"vEmpty{sv}"].arrive()
            else:
                pending = sv
        if pending >= 0:
            bars[f"vEmpty{pending}"].arrive()

    def tile_warp(w):
        x_uses = [0]

        def im2col(t):
            if w == 0:
                yield from wait("stFull", t)
            yield from barsync(4)
            if w == 0 and t > 0:
                yield from wait("imEmpty", t - 1)
            yield from barsync(4)
            yield from barsync(4)
            if w == 0:
                bars["imFull"].arrive()
                bars["stEmpty"].arrive()

        def fold(t):
            yield from barsync(4)
            if w == 0:
                async_q.append("xFull")
                yield from wait("xFull", x_uses[0])
                x_uses[0] += 1
                yield from wait("d2Full", t)
            yield from barsync(4)
            for r in range(16):
                if r == 12:
                    bars["d2Empty"].arrive()
                yield from barsync(4)
            yield from barsync(4)
            if w == 0:
                bars["foldFree"].arrive()

        if tiles == 0:
            return
        yield from im2col(0)
        for t in range(tiles):
            if t + 1 < tiles:
                yield from im2col(t + 1)
            yield from fold(t)

    roles = {"wload": weight_loader(), "vload": v_stage_loader(), "mma": mma()}
    for w in range(16):
        roles[f"epi{w}"] = epilogue(w)
    for w in range(4):
        roles[f"tile{w}"] = tile_warp(w)
    finished = set()
    for _ in range(max_steps):
        choices = [k for k in roles if k not in finished]
        if async_q:
            choices.append("async")
        if commit_q:
            choices.append("commit")
        rnd.shuffle(choices)
        progressed = False
        blocked = []
        for c in choices:
            if c == "async":
                bars[async_q.pop(rnd.randrange(len(async_q)))].arrive()
                progressed = True
                break
            if c == "commit":
                bars[commit_q.pop(0)].arrive()
                progressed = True
                break
            before = (clock[0], len(async_q), len(commit_q))
            try:
                r = next(roles[c])
            except StopIteration:
                finished.add(c)
                progressed = True
                break
            if r == "blocked" and (clock[0], len(async_q), len(commit_q)) == before:
                blocked.append(c)
                continue
            progressed = True
            break
        if len(finished) == len(roles) and not async_q and not commit_q:
            open_phases = [n for n, b in bars.items() if b.pending]
            if open_phases:
                return f"barriers left mid-phase: {open_phases}"
            return "ok" if not hazards else f"parity aliasing: {hazards[:3]}"
        if not progressed:
            return f"deadlock: {sorted(blocked)}" + (f"; parity aliasing: {hazards[:3]}" if hazards else "")
    return "no end within the step limit"


@pytest.mark.parametrize("n_blk", [1, 2, 3, 4, 8])
@pytest.mark.parametrize("n_v", [2, 4])
def test_kernel_f_protocol_every_shape(n_blk, n_v):
    """Every V ring the solver accepts (2, 4), weight rings 2-4, tiles of 1-8 64-feature
    blocks, 0-5 tiles per CTA, several schedules each."""
    for n_w in (2, 3, 4):
        for tiles in (0, 1, 2, 3, 5):
            for seed in range(3):
                r = run_protocol(n_blk, n_v, n_w, tiles, seed)
                assert r == "ok", (n_blk, n_v, n_w, tiles, seed, r)


def test_shared_single_v_slot_is_caught():
    """One V slot shared by the two epilogue groups: a group can test the slot's parity while
    the barrier is two phases ahead of the use it waits for (parity aliasing), or both groups
    stall; the model flags it.  The kernel gives each group its own slots (even rings, group g
    taking slots g, g + 2, ...)."""
    found = [run_protocol(n_blk, 1, n_w, tiles, seed)
             for n_blk in (2, 4) for n_w in (2, 3) for tiles in (2, 3) for seed in range(3)]
    assert any(r != "ok" for r in found), found
