"""CPU model check of the mbarrier protocols of the persistent tensor-core kernels: the LCA
solver's reconstruction kernel R (recon_tc_kernel), post-delivery + update kernel P
(post_tc_kernel) and fused timestep kernel F (step_tc_kernel) in openpv_gb300/csrc/lca_solver.cu,
and the tensor-core delivery (conv_tf32x3_kernel) in openpv_gb300/csrc/deliver_tc.cu.

Every role of one CTA runs as a coroutine over exact mbarrier semantics (a wait for phase k
tests parity k & 1 and passes once the barrier has completed a phase of the other parity; a
barrier completes a phase when its expected arrivals are in) and named barriers (all member
warps arrive, then all pass).  A random scheduler interleaves the roles with the completions of
asynchronous copies (TMA / bulk loads, in any order) and of tcgen05 commits (in issue order).  A
run passes when every role finishes, every mbarrier ends on a phase boundary and no wait ever
observed a barrier more than one phase away from the phase it waits for (parity aliasing).  The
models follow the kernels' loops and name the barriers as the kernels do.
"""
import random

import pytest


class _Sim:
    def __init__(self, seed):
        self.rnd = random.Random(seed)
        self.clock = 0
        self.hazards = []
        self.count, self.pending, self.done = {}, {}, {}
        self.async_q, self.commit_q = [], []
        self.named = {}

    def mk(self, name, count=1):
        self.count[name], self.pending[name], self.done[name] = count, 0, 0

    def arrive(self, name):
        self.clock += 1
        self.pending[name] += 1
        assert self.pending[name] <= self.count[name], f"more arrivals at {name} than it expects"
        if self.pending[name] == self.count[name]:
            self.pending[name] = 0
            self.done[name] += 1

    def test(self, name, k):
        d = self.done[name]
        if d < k or d > k + 1:
            self.hazards.append((name, k, d))
        return (d & 1) != (k & 1)

    def wait(self, name, k):
        while not self.test(name, k):
            yield "blocked"

    def barsync(self, bid, n):
        st = self.named.setdefault(bid, [0, 0])
        gen = st[1]
        st[0] += 1
        self.clock += 1
        if st[0] == n:
            st[0] = 0
            st[1] += 1
        while self.named[bid][1] == gen:
            yield "blocked"

    def run(self, roles, max_steps=2_000_000):
        finished = set()
        for _ in range(max_steps):
            choices = [k for k in roles if k not in finished]
            if self.async_q:
                choices.append("async")
            if self.commit_q:
                choices.append("commit")
            self.rnd.shuffle(choices)
            progressed = False
            blocked = []
            for c in choices:
                if c == "async":
                    self.arrive(self.async_q.pop(self.rnd.randrange(len(self.async_q))))
                    progressed = True
                    break
                if c == "commit":
                    self.arrive(self.commit_q.pop(0))
                    progressed = True
                    break
                before = (self.clock, len(self.async_q), len(self.commit_q))
                try:
                    r = next(roles[c])
                except StopIteration:
                    finished.add(c)
                    progressed = True
                    break
                if r == "blocked" and (self.clock, len(self.async_q), len(self.commit_q)) == before:
                    blocked.append(c)
                    continue
                progressed = True
                break
            if len(finished) == len(roles) and not self.async_q and not self.commit_q:
                open_phases = [n for n, p in self.pending.items() if p]
                if open_phases:
                    return f"barriers left mid-phase: {open_phases}"
                return "ok" if not self.hazards else f"parity aliasing: {self.hazards[:3]}"
            if not progressed:
                return f"deadlock: {sorted(blocked)}" + (f"; parity aliasing: {self.hazards[:3]}" if self.hazards else "")
        return "no end within the step limit"


# ---------------------------------------------------------------------------------------------
# kernel R: load warp, MMA warp, 8 fold warps (named barrier 1)
# ---------------------------------------------------------------------------------------------
def run_kernel_r(units, n_mb, nkc, n_stage, seed):
    """units: images of this CTA; n_mb: 128-position blocks per image; nkc: 64-feature chunks."""
    s = _Sim(seed)
    for i in range(n_stage):
        s.mk(f"full{i}")
        s.mk(f"empty{i}")
    for i in range(2):
        s.mk(f"accFull{i}")
        s.mk(f"accEmpty{i}", 8)
        s.mk(f"xFull{i}")
        s.mk(f"xEmpty{i}")

    def loads():
        j = 0
        for ui in range(units):
            for mb in range(n_mb):
                for _ in range(nkc):
                    st, u = j % n_stage, j // n_stage
                    if u > 0:
                        yield from s.wait(f"empty{st}", u - 1)
                    s.async_q.append(f"full{st}")  # the A tile and the W^T tile of the stage
                    j += 1
                    yield "step"
                if mb == 0:  # the image's x, once the residual of unit ui - 2 has read its buffer
                    xb = ui & 1
                    if ui >= 2:
                        yield from s.wait(f"xEmpty{xb}", (ui >> 1) - 1)
                    s.async_q.append(f"xFull{xb}")
                    yield "step"

    def mma():
        j = blk = 0
        for _ in range(units):
            for _ in range(n_mb):
                a = blk & 1
                if blk >= 2:
                    yield from s.wait(f"accEmpty{a}", (blk >> 1) - 1)
                for _ in range(nkc):
                    yield from s.wait(f"full{j % n_stage}", j // n_stage)
                    s.commit_q.append(f"empty{j % n_stage}")
                    j += 1
                    yield "step"
                s.commit_q.append(f"accFull{a}")
                blk += 1

    def fold(w):
        blk = 0
        yield from s.barsync(1, 8)  # the image buffer cleared
        for ui in range(units):
            for _ in range(n_mb):
                a = blk & 1
                if w == 0:
                    yield from s.wait(f"accFull{a}", blk >> 1)
                yield from s.barsync(1, 8)
                for ty in range(4):  # tap rows, four tap columns each, one barrier per group
                    if ty == 3:
                        s.arrive(f"accEmpty{a}")  # this warp has read the accumulator
                    for _ in range(4):
                        yield from s.barsync(1, 8)
                blk += 1
            xb = ui & 1
            if w == 0:
                yield from s.wait(f"xFull{xb}", ui >> 1)
            yield from s.barsync(1, 8)
            yield from s.barsync(1, 8)  # the residual written
            if w == 0:
                s.arrive(f"xEmpty{xb}")
            yield from s.barsync(1, 8)  # the image buffer cleared again

    roles = {"loads": loads(), "mma": mma()}
    for w in range(8):
        roles[f"fold{w}"] = fold(w)
    return s.run(roles)


# ---------------------------------------------------------------------------------------------
# kernel P: load warp, MMA warp (4 accumulators), 8 epilogue warps (named barrier 1)
# ---------------------------------------------------------------------------------------------
def run_kernel_p(n_blk, n_v, n_w, tiles, seed, k_im=None):
    """n_blk: 64-feature blocks per tile; tiles: tiles of this CTA; k_im: the block after which
    the next tile's im2col runs (None: the kernel's choice)."""
    s = _Sim(seed)
    q_total = n_blk * tiles
    for n in ("stFull", "stEmpty", "imFull", "imEmpty"):
        s.mk(n)
    for i in range(n_w):
        s.mk(f"wFull{i}")
        s.mk(f"wEmpty{i}")
    for i in range(n_v):
        s.mk(f"vFull{i}")
        s.mk(f"vEmpty{i}", 8)
    for i in range(4):
        s.mk(f"accFull{i}")
        s.mk(f"accEmpty{i}", 8)
    lag_v = n_v - 1 if n_v >= 2 else n_v
    if k_im is None:
        k_im = min(max(n_blk - 1 - lag_v, 1), n_blk - 1)

    def loads():
        rows = 0
        if tiles == 0:
            return
        s.async_q.append("stFull")  # tile 0's residual window
        rows = 1
        sw = uw = sv = uv = 0
        for q in range(q_total):
            # tile t+1's window once tile t's has been read, before the first load that waits
            # for tile t's epilogue or MMAs
            while rows < tiles and (rows - 1) * n_blk + min(lag_v, n_w) <= q:
                yield from s.wait("stEmpty", rows - 1)
                s.async_q.append("stFull")
                rows += 1
            if uw > 0:
                yield from s.wait(f"wEmpty{sw}", uw - 1)
            s.async_q.append(f"wFull{sw}")
            if uv > 0:
                yield from s.wait(f"vEmpty{sv}", uv - 1)
            s.async_q.append(f"vFull{sv}")
            yield "step"
            sw += 1
            if sw == n_w:
                sw, uw = 0, uw + 1
            sv += 1
            if sv == n_v:
                sv, uv = 0, uv + 1
        while rows < tiles:
            yield from s.wait("stEmpty", rows - 1)
            s.async_q.append("stFull")
            rows += 1

    def mma():
        sw = uw = nb = ti = 0
        for q in range(q_total):
            a = q % 4
            if nb == 0:
                yield from s.wait("imFull", ti)
            yield from s.wait(f"wFull{sw}", uw)
            if q >= 4:
                yield from s.wait(f"accEmpty{a}", q // 4 - 1)
            s.commit_q.append(f"accFull{a}")
            s.commit_q.append(f"wEmpty{sw}")
            if nb == n_blk - 1:
                s.commit_q.append("imEmpty")
            yield "step"
            sw += 1
            if sw == n_w:
                sw, uw = 0, uw + 1
            nb += 1
            if nb == n_blk:
                nb, ti = 0, ti + 1

    def epilogue(w):
        def im2col(t):
            if w == 0:
                yield from s.wait("stFull", t)
                if t > 0:
                    yield from s.wait("imEmpty", t - 1)  # the previous tile's MMAs are done
            yield from s.barsync(1, 8)
            yield from s.barsync(1, 8)
            if w == 0:
                s.arrive("imFull")
                s.arrive("stEmpty")

        if tiles == 0:
            return
        yield from im2col(0)
        pending = -1
        sv = uv = nb = ti = 0
        for q in range(q_total):
            a = q % 4
            yield from s.wait(f"accFull{a}", q // 4)
            yield from s.wait(f"vFull{sv}", uv)
            s.arrive(f"accEmpty{a}")
            yield "step"  # the update
            if pending >= 0:
                s.arrive(f"vEmpty{pending}")  # the previous store has read its slot
            yield "step"  # the V (and A) stores
            if n_v == 1:
                s.arrive(f"vEmpty{sv}")
                pending = -1
            else:
                pending = sv
            if nb == k_im and ti + 1 < tiles:
                yield from im2col(ti + 1)
            sv += 1
            if sv == n_v:
                sv, uv = 0, uv + 1
            nb += 1
            if nb == n_blk:
                nb, ti = 0, ti + 1

    roles = {"loads": loads(), "mma": mma()}
    for w in range(8):
        roles[f"epi{w}"] = epilogue(w)
    return s.run(roles)


# ---------------------------------------------------------------------------------------------
# kernel F: weight loads, event-loop V/stage loads, event-loop MMA, two epilogue groups of 8
# warps on alternating blocks (no named barrier), 4 tile warps (named barrier 1)
# ---------------------------------------------------------------------------------------------
def run_kernel_f(n_blk, n_v, n_w, tiles, seed, group_slots=True):
    """group_slots: V slots as the kernel assigns them (group g takes slots g, g + 2, ...); with
    False the two groups share the ring in block order (a shape the kernel does not use)."""
    s = _Sim(seed)
    q_total = tiles * n_blk
    for n in ("stFull", "stEmpty", "imFull", "imEmpty", "d2Full", "foldFree", "xFull"):
        s.mk(n)
    s.mk("d2Empty", 4)
    for i in range(n_w):
        s.mk(f"wFull{i}")
        s.mk(f"wEmpty{i}")
    for i in range(n_v):
        s.mk(f"vFull{i}")
        s.mk(f"vEmpty{i}", 8)
    for i in range(2):
        s.mk(f"accFull{i}")
        s.mk(f"accEmpty{i}", 8)
        s.mk(f"aFull{i}", 8)
        s.mk(f"aEmpty{i}")

    def weight_loader():  # per block: wEmpty[slot] (previous use) -> wFull[slot]
        sw = uw = 0
        for _ in range(q_total):
            if uw > 0:
                yield from s.wait(f"wEmpty{sw}", uw - 1)
            s.async_q.append(f"wFull{sw}")
            yield "step"
            sw += 1
            if sw == n_w:
                sw, uw = 0, uw + 1

    def v_stage_loader():  # event loop: the next tile's stage; the next block's V chunk
        st_next = vq = sv = uv = 0
        while st_next < tiles or vq < q_total:
            did = False
            if st_next < tiles and (st_next == 0 or s.test("stEmpty", st_next - 1)) and \
                    (st_next < 2 or s.test("foldFree", st_next - 2)):
                s.async_q.append("stFull")
                st_next += 1
                did = True
            if vq < q_total and (uv == 0 or s.test(f"vEmpty{sv}", uv - 1)):
                s.async_q.append(f"vFull{sv}")
                vq += 1
                did = True
                sv += 1
                if sv == n_v:
                    sv, uv = 0, uv + 1
            yield "step" if did else "blocked"

    def mma():  # event loop: GEMM1 and GEMM2 of successive blocks
        g1 = ti1 = nb1 = sw1 = uw1 = 0
        g2 = nb2 = sw2 = ti2 = 0
        while g2 < q_total:
            did = False
            if g1 < q_total:
                a = g1 & 1
                if (nb1 != 0 or s.test("imFull", ti1)) and s.test(f"wFull{sw1}", uw1) and \
                        (g1 < 2 or s.test(f"accEmpty{a}", g1 // 2 - 1)):
                    s.commit_q.append(f"accFull{a}")
                    if nb1 == n_blk - 1:
                        s.commit_q.append("imEmpty")
                    g1 += 1
                    sw1 += 1
                    if sw1 == n_w:
                        sw1, uw1 = 0, uw1 + 1
                    nb1 += 1
                    if nb1 == n_blk:
                        nb1, ti1 = 0, ti1 + 1
                    did = True
            if g2 < g1 and s.test(f"aFull{g2 & 1}", g2 >> 1) and \
                    (nb2 != 0 or ti2 == 0 or s.test("d2Empty", ti2 - 1)):
                s.commit_q.append(f"aEmpty{g2 & 1}")
                s.commit_q.append(f"wEmpty{sw2}")
                if nb2 == n_blk - 1:
                    s.commit_q.append("d2Full")
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
        sv, uv = g, 0
        for q in range(g, q_total, 2):
            k = q >> 1
            if not group_slots:
                sv, uv = q % n_v, q // n_v
            if pending >= 0:  # the V slot of the group's previous block
                s.arrive(f"vEmpty{pending}")
                pending = -1
            yield from s.wait(f"accFull{g}", k)
            yield from s.wait(f"vFull{sv}", uv)
            s.arrive(f"accEmpty{g}")
            yield "step"  # the update
            if k >= 1:
                yield from s.wait(f"aEmpty{g}", k - 1)
            s.arrive(f"aFull{g}")
            yield "step"  # the V store
            if n_v == 2:
                s.arrive(f"vEmpty{sv}")
            else:
                pending = sv
            if group_slots:
                sv += 2
                if sv >= n_v:
                    sv, uv = g, uv + 1
        if pending >= 0:
            s.arrive(f"vEmpty{pending}")

    def tile_warp(w):
        x_uses = 0

        def im2col(t):
            if w == 0:
                yield from s.wait("stFull", t)
            yield from s.barsync(1, 4)
            if w == 0 and t > 0:
                yield from s.wait("imEmpty", t - 1)
            yield from s.barsync(1, 4)
            yield from s.barsync(1, 4)
            if w == 0:
                s.arrive("imFull")
                s.arrive("stEmpty")

        def fold(t):
            nonlocal x_uses
            yield from s.barsync(1, 4)  # the previous band store has read the buffer
            if w == 0:
                s.async_q.append("xFull")
                yield from s.wait("xFull", x_uses)
                x_uses += 1
                yield from s.wait("d2Full", t)
            yield from s.barsync(1, 4)
            for r in range(16):  # tap groups; D2 released after the last TMEM load
                if r == 12:
                    s.arrive("d2Empty")
                yield from s.barsync(1, 4)
            yield from s.barsync(1, 4)
            if w == 0:
                s.arrive("foldFree")

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
    return s.run(roles)


# ---------------------------------------------------------------------------------------------
# the tensor-core delivery (conv_tf32x3_kernel, openpv_gb300/csrc/deliver_tc.cu): TMA producer,
# MMA issuer, 4 split warps (each on its own), 4 epilogue warps (each on its own)
# ---------------------------------------------------------------------------------------------
def run_conv_tc(R, NS, NR, NB, KX, KY, nFC, units, seed):
    """R target rows per unit, NS split-row slots, NR raw-row slots, NB weight-tile slots,
    KX x KY patch, nFC 32-feature source chunks, units of this CTA."""
    s = _Sim(seed)
    for i in range(NR):
        s.mk(f"rawFull{i}")
        s.mk(f"rawEmpty{i}", 4)
    for i in range(NS):
        s.mk(f"aReady{i}", 4)
        s.mk(f"aEmpty{i}")
    for i in range(NB):
        s.mk(f"bFull{i}")
        s.mk(f"bEmpty{i}")
    for i in range(2):
        s.mk(f"chainFull{i}")
        s.mk(f"chainEmpty{i}", 4)
    rows_per_fc = R + KY - 1
    groups_per_unit = nFC * KY
    groups_per_chain = max(1, min(KY, (7 + KX - 1) // KX))
    chains_per_unit = (groups_per_unit + groups_per_chain - 1) // groups_per_chain

    def producer():
        ca = cb = 0
        for _ in range(units):
            for _ in range(nFC):
                def load_a():
                    nonlocal ca
                    rr = ca % NR
                    if ca >= NR:
                        yield from s.wait(f"rawEmpty{rr}", ca // NR - 1)
                    s.async_q.append(f"rawFull{rr}")
                    ca += 1
                    yield "step"

                def load_b():
                    nonlocal cb
                    d = cb % NB
                    if cb >= NB:
                        yield from s.wait(f"bEmpty{d}", cb // NB - 1)
                    s.async_q.append(f"bFull{d}")  # the hi and lo weight rows
                    cb += 1
                    yield "step"

                for _ in range(R - 1):
                    yield from load_a()
                for _ in range(KY):
                    yield from load_a()
                    for _ in range(KX):
                        yield from load_b()

    def mma():
        cbase = cb = cc = 0
        slot_base = 0
        for _ in range(units):
            grp = 0
            for _ in range(nFC):
                for ky in range(KY):
                    if grp % groups_per_chain == 0 and cc >= 2:
                        yield from s.wait(f"chainEmpty{cc & 1}", (cc >> 1) - 1)
                    for j in range(0 if ky == 0 else ky + R - 1, ky + R):
                        c = cbase + j
                        yield from s.wait(f"aReady{c % NS}", c // NS)
                    slot_ky = (slot_base + ky) % NS
                    for _ in range(KX):
                        yield from s.wait(f"bFull{cb % NB}", cb // NB)
                        s.commit_q.append(f"bEmpty{cb % NB}")
                        cb += 1
                        yield "step"
                    s.commit_q.append(f"aEmpty{slot_ky}")  # row ky has no later use
                    if (grp + 1) % groups_per_chain == 0 or grp + 1 == groups_per_unit:
                        s.commit_q.append(f"chainFull{cc & 1}")
                        cc += 1
                    grp += 1
                for j in range(KY, rows_per_fc):
                    s.commit_q.append(f"aEmpty{(slot_base + j) % NS}")
                cbase += rows_per_fc
                slot_base = (slot_base + rows_per_fc) % NS

    def split(w):
        c = 0
        for _ in range(units):
            for _ in range(nFC):
                for _ in range(rows_per_fc):
                    rr, sl = c % NR, c % NS
                    yield from s.wait(f"rawFull{rr}", c // NR)
                    if c >= NS:
                        yield from s.wait(f"aEmpty{sl}", c // NS - 1)
                    yield "step"  # hi / lo split of the row
                    s.arrive(f"aReady{sl}")
                    s.arrive(f"rawEmpty{rr}")
                    c += 1

    def epilogue(w):
        cc = 0
        for _ in range(units):
            for _ in range(chains_per_unit):
                yield from s.wait(f"chainFull{cc & 1}", cc >> 1)
                yield "step"  # the chain's sums
                s.arrive(f"chainEmpty{cc & 1}")
                cc += 1

    roles = {"tma": producer(), "mma": mma()}
    for w in range(4):
        roles[f"split{w}"] = split(w)
        roles[f"epi{w}"] = epilogue(w)
    return s.run(roles)


# ---------------------------------------------------------------------------------------------
@pytest.mark.parametrize("n_stage", [2, 3, 4])
def test_kernel_r_protocol(n_stage):
    """Kernel R: every ring depth the solver uses, 1-2 position blocks per image, 0-5 images
    per CTA (x double-buffered across them)."""
    for units in (0, 1, 2, 3, 5):
        for n_mb in (1, 2):
            for nkc in (1, 4, 8):
                for seed in range(3):
                    r = run_kernel_r(units, n_mb, nkc, n_stage, seed)
                    assert r == "ok", (units, n_mb, nkc, n_stage, seed, r)


@pytest.mark.parametrize("n_v", [1, 2, 3])
def test_kernel_p_protocol(n_v):
    """Kernel P: V rings 1-3, weight rings 1-2, feature tiles of 1-4 blocks, 0-5 tiles per CTA,
    the next tile's im2col inside the current tile's block loop where the kernel puts it."""
    for n_w in (1, 2):
        for n_blk in (1, 2, 3, 4):
            for tiles in (0, 1, 2, 3, 5):
                for seed in range(3):
                    r = run_kernel_p(n_blk, n_v, n_w, tiles, seed)
                    assert r == "ok", (n_blk, n_v, n_w, tiles, seed, r)


@pytest.mark.parametrize("n_blk", [1, 2, 3, 4, 8])
@pytest.mark.parametrize("n_v", [2, 4])
def test_kernel_f_protocol(n_blk, n_v):
    """Kernel F: every V ring the solver accepts (2, 4), weight rings 2-4, feature tiles of 1-8
    blocks, 0-5 tiles per CTA."""
    for n_w in (2, 3, 4):
        for tiles in (0, 1, 2, 3, 5):
            for seed in range(3):
                r = run_kernel_f(n_blk, n_v, n_w, tiles, seed)
                assert r == "ok", (n_blk, n_v, n_w, tiles, seed, r)


def test_kernel_f_shared_v_slot_is_caught():
    """The two epilogue groups sharing one V slot: a group can test the slot's parity while the
    barrier is two phases ahead of the use it waits for, or both groups stall; the model flags
    it.  The kernel gives each group its own slots (even rings, group g taking g, g + 2, ...)."""
    found = [run_kernel_f(n_blk, 1, n_w, tiles, seed, group_slots=False)
             for n_blk in (2, 4) for n_w in (2, 3) for tiles in (2, 3) for seed in range(3)]
    assert any(r != "ok" for r in found), found


def test_kernel_p_early_im2col_is_caught():
    """Kernel P places the next tile's im2col no earlier than block 1 of a multi-block tile:
    after block 0, with one V slot and one weight slot, the im2col's wait for the tile's last MMA
    stalls the epilogue that those MMAs' loads wait for, and the model finds the deadlock."""
    found = [run_kernel_p(4, 1, 1, 2, seed, k_im=0) for seed in range(4)]
    assert any(r.startswith("deadlock") for r in found), found
    assert all(run_kernel_p(4, 1, 1, 2, seed) == "ok" for seed in range(4))


@pytest.mark.parametrize("R", [1, 2, 3, 4])
def test_conv_tc_protocol(R):
    """The tensor-core delivery: split-row rings of R + 1 and R + 2 slots, one or two raw rows,
    2-8 weight-tile slots, patches of 1x1 to 9x9, 1-3 source chunks, 0-3 units per CTA."""
    for NS in (R + 1, R + 2):
        for NR in (1, 2):
            for NB in (2, 3, 8):
                for KX, KY in ((1, 1), (3, 3), (7, 7), (9, 5)):
                    for nFC in (1, 3):
                        for units in (0, 1, 3):
                            r = run_conv_tc(R, NS, NR, NB, KX, KY, nFC, units, seed=R + NS + NB + KX + units)
                            assert r == "ok", (R, NS, NR, NB, KX, KY, nFC, units, r)
