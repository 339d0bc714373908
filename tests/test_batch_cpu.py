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
