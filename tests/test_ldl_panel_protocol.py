"""CPU model of the panel broadcast protocol of the cluster LDL^T kernel
(k_global_ldl_panel in thesis-emx-bach_gb300/csrc/xb_ldl.cu).

The cluster factors panels of P columns; panel p belongs to CTA p % CL,
which factors it (after the updates of every earlier panel) and copies it to
ring slot p % RING of every other CTA with one bulk copy per receiver,
completing on the receiver's "full" mbarrier of that slot.  A receiver arms
the slot (arrive.expect_tx) before the copy can come, reads the panel, applies
it, re-arms the slot for the next panel it will receive there and arrives on
the "empty" mbarrier of the CTA that sends panel p + RING, which waits for
CL - 1 such arrivals before its copy.  The owner of panel p + 1 applies panel
p to it first and sends it before updating its other columns (look-ahead).

This model runs the protocol as interleaved per-CTA actions (random
schedules, many seeds) with the mbarrier rules of the PTX ISA (pending
arrivals, a signed transaction count, phases with parity waits) and checks
that it never deadlocks, that no copy lands in a slot whose previous panel a
receiver still reads, that every panel is read after its copy completed, and
that every CTA sees panels in order.  No GPU is involved.
"""
import random

import pytest


class MBar:
    def __init__(self, count):
        self.count = count
        self.pending = count
        self.tx = 0
        self.phase = 0

    def _maybe_complete(self):
        if self.pending == 0 and self.tx == 0:
            self.phase += 1
            self.pending = self.count

    def arrive(self):
        self.pending -= 1
        assert self.pending >= 0, "arrival beyond the expected count"
        self._maybe_complete()

    def arrive_expect(self, nbytes):
        self.tx += nbytes
        self.arrive()

    def complete_tx(self, nbytes):
        self.tx -= nbytes
        self._maybe_complete()

    def done(self, parity):
        # try_wait.parity(parity) succeeds once the phase of that parity completed
        return (self.phase & 1) != parity


def run(n_panels, CL, RING, seed):
    assert RING <= CL
    rng = random.Random(seed)
    owner = lambda p: p % CL
    last_sent = n_panels - 2  # the last panel updates nothing: it is not sent
    NB = 1000  # bytes per panel copy (any positive size)
    full = [[MBar(1) for _ in range(RING)] for _ in range(CL)]
    empty = [MBar(CL - 1) for _ in range(CL)]
    slot_panel = [[None] * RING for _ in range(CL)]   # panel whose data sits in the slot
    slot_busy = [[False] * RING for _ in range(CL)]   # a receiver is reading it
    consumed = [set() for _ in range(CL)]

    def receives(r, p):
        return owner(p) != r and p <= last_sent

    # arm each slot for the first panel received through it
    for r in range(CL):
        for s in range(RING):
            for p in range(s, last_sent + 1, RING):
                if receives(r, p):
                    full[r][s].arrive_expect(NB)
                    break

    def sender(r):
        # the sequence of actions of CTA r, as a generator of (kind, payload)
        phase_bits = 0
        empty_phase = 0

        def send(p):
            nonlocal empty_phase
            if p >= RING:
                while not empty[r].done(empty_phase):
                    yield ("wait", None)
                empty_phase ^= 1
            s = p % RING
            for q in range(CL):
                if q == r:
                    continue
                assert not slot_busy[q][s], f"panel {p} overwrites slot {s} of CTA {q} in use"
                prev = slot_panel[q][s]
                if prev is not None and receives(q, prev):
                    assert prev in consumed[q], f"panel {prev} in CTA {q} overwritten unread"
                slot_panel[q][s] = p
                full[q][s].complete_tx(NB)
                yield ("step", None)

        if owner(0) == r and 0 <= last_sent:
            yield from send(0)
        for p in range(0, n_panels - 1):
            s = p % RING
            own = owner(p) == r
            if not own:
                while not full[r][s].done((phase_bits >> s) & 1):
                    yield ("wait", None)
                phase_bits ^= 1 << s
                assert slot_panel[r][s] == p, f"CTA {r} reads panel {slot_panel[r][s]} for {p}"
                slot_busy[r][s] = True
            if owner(p + 1) == r and p + 1 <= last_sent:
                yield from send(p + 1)
            yield ("step", None)  # trailing update (reads the slot)
            if not own:
                slot_busy[r][s] = False
                consumed[r].add(p)
                for pn in range(p + RING, last_sent + 1, RING):
                    if receives(r, pn):
                        full[r][s].arrive_expect(NB)
                        break
                if p + RING <= last_sent:
                    empty[owner(p + RING)].arrive()
            yield ("step", None)

    gens = [sender(r) for r in range(CL)]
    alive = set(range(CL))
    stalled = 0
    while alive:
        r = rng.choice(sorted(alive))
        try:
            kind, _ = next(gens[r])
        except StopIteration:
            alive.discard(r)
            stalled = 0
            continue
        stalled = stalled + 1 if kind == "wait" else 0
        assert stalled < 200 * CL, "no CTA can make progress: deadlock"
    for r in range(CL):
        want = {p for p in range(n_panels - 1) if receives(r, p)}
        assert consumed[r] == want


@pytest.mark.parametrize("n_panels,CL,RING", [(37, 16, 4), (37, 16, 2), (74, 16, 4), (147, 16, 2),
                                              (19, 8, 8), (5, 16, 4), (2, 16, 4), (1, 16, 4),
                                              (40, 8, 3)])
def test_panel_ring_protocol(n_panels, CL, RING):
    for seed in range(60):
        run(n_panels, CL, RING, seed)
