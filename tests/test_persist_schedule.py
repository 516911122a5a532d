"""The work-queue schedules of the persistent Richardson-Lucy kernels, restated in Python and
run as a discrete-event simulation with random item durations and CTA counts.

* Single volume (iane_gb300/csrc/rl_persist.cuh): phase 2t = pass A of iteration t (reads the
  estimate with a halo of rz planes, writes the ratio), 2t + 1 = pass B (reads the ratio with
  the halo, reads and rewrites its own estimate planes). Items are (phase, z, tile) in that
  order; an item of phase p at plane z starts once planes z - rz .. z + rz have completed
  p * tiles items (per-plane counters).
* Batch (iane_gb300/csrc/rl_batch_kernel.cu): items (phase, image, tile); an item of phase p
  starts once its image has completed p * tiles items.

The simulation takes items in queue order into free CTAs, starts an item when its counter rule
holds, and checks at every start and finish that the rule really orders the data: every plane
an item reads holds the previous phase's result (read after write), no item overwrites a plane
that an item of the previous phase is still reading (write after read), a counter that reached
p * tiles means phases < p are complete on that plane, and the run never stalls (progress).
With per-iteration statistics the volume's pass B items also write partials into a buffer per
iteration parity, combined when an iteration's last pass B item finishes: no partial is
overwritten before its iteration is combined, and iterations are combined in order."""
from __future__ import annotations

import heapq
import random

import pytest


def simulate(items, ready, reads, writes, finish, ctas, seed):
    """items: queue order; ready(item): the counter rule; reads(item): {(buffer, plane): phase
    of the writer whose value the item must read} over its run; writes(item): (buffer, plane)
    written at its end; finish(item): counter update. Returns the completion order; raises
    AssertionError on a hazard or a stall."""
    rng = random.Random(seed)
    version = {}              # (buffer, plane) -> phase of the last writer (-1: the start values)
    active_reads = {}         # (buffer, plane) -> count of running readers, by the reader's phase
    head = 0
    holding = [None] * ctas   # item held by each CTA (taken, not started)
    running = []              # heap of (end time, seq, cta, item)
    seq = 0
    now = 0.0
    done = []
    while head < len(items) or any(h is not None for h in holding) or running:
        progressed = False
        for c in range(ctas):
            if holding[c] is None and head < len(items) and not any(r[2] == c for r in running):
                holding[c] = items[head]
                head += 1
                progressed = True
        for c in range(ctas):
            it = holding[c]
            if it is not None and ready(it):
                for key, want in reads(it).items():
                    # read after write: the value of the expected writer is there
                    assert version.get(key, -1) == want, (it, key, version.get(key), want)
                    active_reads[key] = active_reads.get(key, 0) + 1
                end = now + rng.uniform(0.5, 3.0)
                heapq.heappush(running, (end, seq, c, it))
                seq += 1
                holding[c] = None
                progressed = True
        if not running:
            assert progressed, "stall: no item can start and none is running"
            continue
        end, _, c, it = heapq.heappop(running)
        now = end
        for key in reads(it):
            active_reads[key] -= 1
        for key in writes(it):
            # write after read: nobody still reads the value being replaced
            assert active_reads.get(key, 0) == 0, (it, key)
            version[key] = it[0]
        finish(it)
        done.append(it)
    return done


def volume_case(nz, kz, tiles, phases, ctas, seed, stats=False, stats_wait=True):
    rz = kz // 2
    items = [(p, z, t) for p in range(phases) for z in range(nz) for t in range(tiles)]
    done_count = [0] * nz
    completed = set()
    # statistics: pass B items write partials[parity][item]; the last pass B item of iteration t
    # combines partials[t % 2] when it finishes; pass B of iteration t >= 2 waits for iteration
    # t - 2 to be combined
    per_phase = nz * tiles
    partial_of = {}       # (parity, item index) -> iteration whose partial is stored
    stat_count = [0, 0]
    combined = [0]        # iterations combined so far

    def window(z):
        return range(max(0, z - rz), min(nz, z + rz + 1))

    def ready(it):
        p, z, _ = it
        if stats and stats_wait and p % 2 == 1 and p // 2 >= 2 and combined[0] < p // 2 - 1:
            return False
        return p == 0 or all(done_count[w] >= p * tiles for w in window(z))

    def reads(it):
        # pass A: the estimate (halo) from the previous pass B, or the start values (-1);
        # pass B: the ratio (halo) from pass A, and its own estimate planes from the pass B before
        p, z, t = it
        if p % 2 == 0:
            return {("est", (w, u)): p - 1 for w in window(z) for u in range(tiles)}
        keys = {("ratio", (w, u)): p - 1 for w in window(z) for u in range(tiles)}
        keys[("est", (z, t))] = p - 2 if p >= 2 else -1
        return keys

    def writes(it):
        p, z, t = it
        return {("ratio" if p % 2 == 0 else "est", (z, t))}

    def finish(it):
        p, z, t = it
        if stats and p % 2 == 1:
            n = p // 2
            # the slot may only be overwritten once iteration n - 2 has been combined
            prev = partial_of.get((n % 2, z * tiles + t))
            assert prev is None or prev == n - 2
            assert prev is None or combined[0] >= n - 1
            partial_of[(n % 2, z * tiles + t)] = n
            stat_count[n % 2] += 1
            if stat_count[n % 2] == per_phase:
                # combine: every partial of the parity is this iteration's, and iterations
                # are combined in order
                assert all(partial_of[(n % 2, k)] == n for k in range(per_phase))
                assert combined[0] == n
                stat_count[n % 2] = 0
                combined[0] = n + 1
        done_count[z] += 1
        completed.add(it)
        # a counter that reached q * tiles means phases < q are complete on that plane
        q = done_count[z] // tiles
        assert all((pp, z, u) in completed for pp in range(q) for u in range(tiles))

    out = simulate(items, ready, reads, writes, finish, ctas, seed)
    assert len(out) == len(items)
    if stats:
        assert combined[0] == phases // 2


def batch_case(tiles_per_image, phases, ctas, seed):
    items = [(p, i, t) for p in range(phases) for i, n in enumerate(tiles_per_image) for t in range(n)]
    done_count = [0] * len(tiles_per_image)

    def ready(it):
        p, i, _ = it
        return p == 0 or done_count[i] >= p * tiles_per_image[i]

    def reads(it):
        # as for the volume; a halo may reach any tile of the image
        p, i, t = it
        n = tiles_per_image[i]
        if p % 2 == 0:
            return {("est", (i, u)): p - 1 for u in range(n)}
        keys = {("ratio", (i, u)): p - 1 for u in range(n)}
        keys[("est", (i, t))] = p - 2 if p >= 2 else -1
        return keys

    def writes(it):
        p, i, t = it
        return {("ratio" if p % 2 == 0 else "est", (i, t))}

    def finish(it):
        done_count[it[1]] += 1

    out = simulate(items, ready, reads, writes, finish, ctas, seed)
    assert len(out) == len(items)


@pytest.mark.parametrize("ctas", [1, 2, 5, 16, 200])
@pytest.mark.parametrize("nz,kz,tiles", [(6, 3, 2), (9, 7, 1), (4, 9, 3), (12, 1, 2)])
def test_volume_schedule_orders_every_access(nz, kz, tiles, ctas):
    for seed in range(3):
        volume_case(nz, kz, tiles, phases=6, ctas=ctas, seed=seed)


@pytest.mark.parametrize("ctas", [1, 2, 7, 40, 200])
@pytest.mark.parametrize("nz,kz,tiles", [(6, 3, 2), (9, 7, 1), (2, 5, 3), (20, 1, 1), (24, 3, 1)])
def test_volume_statistics_combine_every_iteration_in_order(nz, kz, tiles, ctas):
    for seed in range(3):
        volume_case(nz, kz, tiles, phases=10, ctas=ctas, seed=seed, stats=True)


def test_statistics_without_their_wait_fail():
    # the checks have teeth: with planes that do not depend on each other (kz = 1), pass B of
    # iteration t + 2 can overwrite a partial before iteration t is combined unless it waits
    with pytest.raises(AssertionError):
        for seed in range(20):
            volume_case(20, 1, 1, phases=10, ctas=200, seed=seed, stats=True, stats_wait=False)


@pytest.mark.parametrize("ctas", [1, 3, 8, 64])
def test_batch_schedule_orders_every_access(ctas):
    for seed in range(3):
        rng = random.Random(seed)
        batch_case([rng.randint(1, 5) for _ in range(7)], phases=6, ctas=ctas, seed=seed)


def test_rule_without_the_halo_fails():
    # the checks have teeth: waiting only for the item's own plane misses the halo's writers
    nz, kz, tiles = 6, 5, 2
    rz = kz // 2
    items = [(p, z, t) for p in range(4) for z in range(nz) for t in range(tiles)]
    done_count = [0] * nz

    def ready(it):
        p, z, _ = it
        return p == 0 or done_count[z] >= p * tiles

    def reads(it):
        p, z, _ = it
        src = "est" if p % 2 == 0 else "ratio"
        return {(src, (w, u)): p - 1 for w in range(max(0, z - rz), min(nz, z + rz + 1)) for u in range(tiles)}

    def writes(it):
        p, z, t = it
        return {("ratio" if p % 2 == 0 else "est", (z, t))}

    def finish(it):
        done_count[it[1]] += 1

    with pytest.raises(AssertionError):
        for seed in range(20):
            simulate(items, ready, reads, writes, finish, ctas=16, seed=seed)
