"""CPU model check of the single-pass compaction's chunk protocol (compact_kernel,
openpv_gb300/csrc/compact.cu): tickets handed out in the order CTAs start (chunk-major: ticket t
is chunk t // nbatch of image t % nbatch), each chunk's total published at once (an aggregate
status), a decoupled look-back over windows of predecessor statuses read one at a time (the
kernel's warp reads 128 per round trip, 4 per lane) back to the nearest published inclusive
prefix, then the chunk's inclusive prefix published.

A random scheduler starts CTAs in any order with at most R resident at a time and interleaves
every status read and publication.  Checked: every run ends (no CTA waits for a chunk whose
CTA cannot run: tickets go to CTAs that have started, so a chunk waits only for chunks of
smaller tickets, whose CTAs are resident or done), and every chunk's exclusive prefix equals the
exclusive scan of its image's chunk totals in chunk order.  Statuses are 0 (not ready),
('agg', total) or ('pre', inclusive), as the kernel's flag bits encode them."""
import random

import pytest


def run_lookback(nbatch, nchunks, resident, window, seed, max_steps=200_000, tickets_at_start=True,
                 stop_at_aggregate=False):
    """tickets_at_start=False gives each CTA the chunk of its launch index instead (the order the
    hardware starts CTAs in is arbitrary); stop_at_aggregate=True ends a look-back at the nearest
    aggregate instead of the nearest inclusive prefix.  Both are shapes the kernel avoids."""
    rnd = random.Random(seed)
    totals = [[rnd.choice((0, 0, 1, 3, 7, 64)) for _ in range(nchunks)] for _ in range(nbatch)]
    status = [[0] * nchunks for _ in range(nbatch)]
    excl_found = {}
    ticket = [0]

    def cta(index):
        if tickets_at_start:
            t = ticket[0]
            ticket[0] += 1
        else:
            t = index
        c, b = t // nbatch, t % nbatch
        total = totals[b][c]
        yield  # the chunk's loads and scans
        st = status[b]
        if c == 0:
            st[0] = ("pre", total)
            excl_found[(b, c)] = 0
            return
        st[c] = ("agg", total)
        excl, j = 0, c - 1
        while True:
            # one round: the window j, j-1, ..., j-window+1 read one status at a time
            seen = []
            for k in range(window):
                idx = j - k
                seen.append(st[idx] if idx >= 0 else ("pre", 0))
                yield
            stops = ("pre", "agg") if stop_at_aggregate else ("pre",)
            first_stop = next((k for k, s in enumerate(seen) if s and s[0] in stops), None)
            upto = seen if first_stop is None else seen[:first_stop + 1]
            if any(s == 0 for s in upto):
                yield  # not ready: read the same window again
                continue
            excl += sum(s[1] for s in upto)
            if first_stop is not None:
                break
            j -= window
        st[c] = ("pre", excl + total)
        excl_found[(b, c)] = excl

    n_ctas = nbatch * nchunks
    waiting = list(range(n_ctas))
    rnd.shuffle(waiting)  # the order the hardware starts CTAs in (blockIdx order does not matter)
    running = []
    for _ in range(max_steps):
        while waiting and len(running) < resident:
            running.append(cta(waiting.pop()))
        if not running:
            break
        g = rnd.choice(running)
        try:
            next(g)
        except StopIteration:
            running.remove(g)
    else:
        return "no end within the step limit"
    for b in range(nbatch):
        acc = 0
        for c in range(nchunks):
            if excl_found.get((b, c)) != acc:
                return f"wrong prefix at image {b} chunk {c}: {excl_found.get((b, c))} != {acc}"
            acc += totals[b][c]
    return "ok"


@pytest.mark.parametrize("resident", [1, 2, 3, 8])
def test_lookback_ends_and_scans(resident):
    for nbatch in (1, 2, 5):
        for nchunks in (1, 2, 7, 20):
            for window in (1, 4):
                for seed in range(4):
                    r = run_lookback(nbatch, nchunks, resident, window, seed)
                    assert r == "ok", (nbatch, nchunks, resident, window, seed, r)


def test_the_model_sees_what_the_kernel_avoids():
    """Chunks bound to launch indices instead of start-order tickets can wait for a chunk whose
    CTA never gets a slot; a look-back that stops at an aggregate adds too little."""
    hung = [run_lookback(2, 6, 1, 4, seed, tickets_at_start=False) for seed in range(6)]
    assert any(r.startswith("no end") for r in hung), hung
    wrong = [run_lookback(2, 6, 3, 4, seed, stop_at_aggregate=True) for seed in range(6)]
    assert any(r.startswith("wrong prefix") for r in wrong), wrong
