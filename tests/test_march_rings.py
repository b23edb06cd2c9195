"""The producer / consumer schedule of the radial-march momentum kernel's two TMA rings (rk_mom_march.cu),
replayed on the CPU for the regular rings (4 halo slots; 3 point slots at the intermediate stages, 2 at the
final one) and the compact rings (3 halo and 2 point slots, issued in the order H0 H1 P0 H2 P1 ...).

The model follows the kernel line by line: the producer issues halo groups H(g) (plane ib-1+g) and point
groups P(m) (level ib+m) in its order, waiting on a slot's "empty" barrier before reusing it; the consumers
wait for H(0) and H(1), release H(0)'s slot, then per level m wait for H(m+2) and P(m), compute, and release
the slots of H(m+1) and P(m). Checked: the schedule finishes for every march depth (no deadlock), every
wait's parity names the use of the slot it waits for, and each group is issued before the consumers reach
the level that needs it, at least a level ahead in the steady state."""
import pytest


def halo_item(n, compact):
    """The kernel's issue order: regular H0 H1 H2 P0 H3 P1 ...; compact H0 H1 P0 H2 P1 H3 P2 ..."""
    if compact:
        return n < 2 or (n >= 3 and (n - 3) % 2 == 0)
    return n < 2 or (n - 2) % 2 == 0


def replay(nlev, nhg, npg, compact):
    total = 2 * nlev + 2
    full = {("h", s): 0 for s in range(nhg)} | {("p", s): 0 for s in range(npg)}     # completed phases
    empty = dict(full)
    issued_at = {}           # item -> consumer position when the producer issued it
    n = gh = gp = 0
    pos = -1                 # consumer: -1 prologue, m = level m, nlev = done
    sc, sn, pn, spc, pp = 1, 2 % nhg, (1 if 2 >= nhg else 0), 0, 0

    def can_issue():
        if n >= total:
            return False
        if halo_item(n, compact):
            s = gh % nhg
            return gh < nhg or empty[("h", s)] >= gh // nhg
        s = gp % npg
        return gp < npg or empty[("p", s)] >= gp // npg

    def issue():
        nonlocal n, gh, gp
        if halo_item(n, compact):
            s = gh % nhg
            full[("h", s)] += 1
            issued_at[("H", gh)] = pos
            gh += 1
        else:
            s = gp % npg
            full[("p", s)] += 1
            issued_at[("P", gp)] = pos
            gp += 1
        n += 1

    def ready(kind, slot, parity):
        # a wait on parity p of a slot passes once the phase it names has completed; the phases a slot has
        # completed count its fills, so the use u (parity u & 1) needs u + 1 completions
        done = full[(kind, slot)]
        assert done <= 2 ** 20
        return done >= 1 and ((done - 1) & 1) == parity

    while True:
        progressed = False
        while can_issue():
            issue()
            progressed = True
        if pos == -1:
            if ready("h", 0, 0) and ready("h", 1, 0):
                empty[("h", 0)] += 1
                pos = 0
                progressed = True
        elif pos < nlev:
            m = pos
            assert sn == (m + 2) % nhg and pn == ((m + 2) // nhg) & 1
            assert spc == m % npg and pp == (m // npg) & 1
            if ready("h", sn, pn) and ready("p", spc, pp):
                # the groups this level reads arrived before the level started
                assert issued_at[("H", m + 2)] < m + 1 or m == 0
                assert issued_at[("P", m)] <= m
                empty[("h", sc)] += 1
                empty[("p", spc)] += 1
                sc = sn
                sn = (sn + 1) % nhg
                if sn == 0:
                    pn ^= 1
                spc = (spc + 1) % npg
                if spc == 0:
                    pp ^= 1
                pos += 1
                progressed = True
        if pos == nlev and n == total:
            return issued_at
        assert progressed, ("deadlock", nlev, nhg, npg, compact, pos, n)


@pytest.mark.parametrize("nhg,npg,compact", [(4, 3, False), (4, 2, False), (3, 2, True)])
@pytest.mark.parametrize("nlev", [1, 2, 3, 4, 5, 13, 20, 39])
def test_ring_schedule_finishes_with_its_groups_ahead(nhg, npg, compact, nlev):
    issued_at = replay(nlev, nhg, npg, compact)
    # the steady-state lead: every point group past the first two is issued while the consumers are at
    # least one level before the level that reads it
    for m in range(2, nlev):
        assert issued_at[("P", m)] <= m - 1, (m, issued_at[("P", m)])
        assert issued_at[("H", m + 2)] <= m, (m, issued_at[("H", m + 2)])


def test_both_issue_orders_keep_a_level_in_flight_with_compact_rings():
    """The release at the end of level m frees the slot of plane m+1 (the level's current plane), so with 3
    halo slots H(m+2) reuses the slot freed when level m-2 ends, and with 2 point slots P(m) the one freed
    when level m-2 ends: the regular order keeps the same one-level lead as the compact order. The compact
    rings' gain is the third block per SM, not the order."""
    for compact in (False, True):
        issued_at = replay(13, 3, 2, compact)
        assert all(issued_at[("P", m)] <= m - 1 for m in range(2, 13))
        assert all(issued_at[("H", m + 2)] <= m for m in range(2, 13))
