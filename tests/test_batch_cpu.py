"""CPU: packing of batched instances into cache-sized block sets."""
from types import SimpleNamespace

from bcmtools_gb300.batch import brick_bytes, chunk_for_cache


class _Tree:
    def __init__(self, nb):
        self.num_leaves = nb


def inst(nb, n=16, vc=1):
    w = SimpleNamespace(tree=_Tree(nb), n=n, vc=vc)
    w.nb = nb
    return w


def test_chunks_keep_order_fit_the_cache_and_isolate_large_instances():
    ws = [inst(nb) for nb in (10, 200, 30, 5000, 40, 40, 1)]
    cache = 3 * 400 * 18 ** 3 * 4  # three fields of 400 blocks of 16^3, vc 1
    chunks = chunk_for_cache(ws, cache)
    assert [w for c in chunks for w in c] == ws  # every instance once, in order
    for c in chunks:
        total = sum(brick_bytes(w) for w in c)
        assert total <= cache or len(c) == 1
    big = [c for c in chunks if any(w.nb == 5000 for w in c)]
    assert big == [[ws[3]]]
    assert chunk_for_cache([], cache) == []


def test_block_sets_pack_small_instances_and_merge_large_ones():
    from bcmtools_gb300.batch import plan_block_sets
    ws = [inst(nb) for nb in (10, 200, 30, 5000, 40, 390, 1, 7000)]
    cache = 3 * 400 * 18 ** 3 * 4
    sets = plan_block_sets(ws, cache)
    flat = [w for s in sets for w in s]
    assert sorted(map(id, flat)) == sorted(map(id, ws))  # every instance once
    assert sets[-1] == [ws[3], ws[7]]  # the instances larger than the cache, together
    for s in sets[:-1]:
        assert sum(brick_bytes(w) for w in s) <= cache
    assert len(sets) == 3  # first-fit decreasing: {390, 10, 1}, {200, 40, 30}, large
    assert plan_block_sets([], cache) == []
    # a cache of fewer than min_set_blocks blocks: one set of everything
    assert plan_block_sets(ws, cache, min_set_blocks=401) == [ws]
    assert len(plan_block_sets(ws, cache, min_set_blocks=400)) == 3
