"""Sharding a batch of independent pivoted QRs across ranks.

A single factorization does not shard (each rank factors its own matrix);
a batch does: matrices are independent, so each rank takes a cost-balanced
subset, factors it with its own GPU (``BatchedQRP``), and the results are
gathered at the end.  There is no collective in the data path -- only the
final gather.
"""


def qr_cost(m, n):
    """Householder QR flops (2 M k^2 - 2 k^3 / 3, k = min(m, n)) plus one pass."""
    M, k = max(m, n), min(m, n)
    return 2.0 * M * k * k - 2.0 * k ** 3 / 3.0 + m * n


def partition_by_cost(shapes, world):
    """Largest-first greedy assignment (LPT) of matrix indices to ranks.

    Returns ``world`` sorted index lists; ties go to the lowest rank, so every
    rank computes the same partition from the same shapes."""
    costs = [qr_cost(m, n) for m, n in shapes]
    order = sorted(range(len(shapes)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def shard_loads(shapes, parts):
    return [sum(qr_cost(*shapes[i]) for i in p) for p in parts]


def gather_to_root(local, indices, world, rank, root=0, group=None):
    """Gather {index: result} from every rank to ``root`` (torch.distributed,
    any backend).  Returns the merged dict on root, None elsewhere."""
    import torch.distributed as dist
    payload = {int(i): r for i, r in zip(indices, local)}
    out = [None] * world if rank == root else None
    dist.gather_object(payload, out, dst=root, group=group)
    if rank != root:
        return None
    merged = {}
    for d in out:
        for k, v in d.items():
            if k in merged:
                raise RuntimeError("matrix %d factored twice" % k)
            merged[k] = v
    return merged
