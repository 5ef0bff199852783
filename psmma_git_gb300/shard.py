"""Row-panel sharding of the structured multiply across ranks (one GPU per rank).

Q[I, :] = alpha * A[I, :] * H + beta * Q[I, :] needs only A's rows I and the O(k)
generators, so the multiply shards by row panels with no exchange on the data path: each
rank multiplies its own panel by the replicated generators.  (For the DFT, where F is on
the left, C[:, J] = F * B[:, J] shards by column panels instead.)  The only collectives are
the ones a caller chooses for timing or for gathering results.
"""
from __future__ import annotations


def panels(n: int, world: int) -> list[tuple[int, int]]:
    """Balanced contiguous [start, stop) panels of range(n) for `world` ranks."""
    if world < 1:
        raise ValueError("world must be >= 1")
    base, extra = divmod(n, world)
    out, s = [], 0
    for r in range(world):
        e = s + base + (1 if r < extra else 0)
        out.append((s, e))
        s = e
    return out


def local_panel(n: int, rank: int, world: int) -> tuple[int, int]:
    return panels(n, world)[rank]


def max_over_ranks(x: float, group=None) -> float:
    """The slowest rank's value (a barrier-synchronised timing is only as fast as it)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size(group) == 1:
        return x
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def sharded_multiply(kind: str, n: int, k: int, alpha, A_panel, gen, beta, Q_panel, *, rank: int, world: int,
                     compute=None, **kw):
    """Computes this rank's row panel Q[I,:] = alpha*A[I,:]*H + beta*Q[I,:] (kind in cauchy,
    toeplitz, hankel).  `A_panel`/`Q_panel` hold rows I = local_panel(n, rank, world);
    `compute` defaults to the library entry point psmma_<kind>."""
    lo, hi = local_panel(n, rank, world)
    rows = hi - lo
    if rows == 0:
        return Q_panel
    if compute is None:
        import psmma_git_gb300 as P
        compute = getattr(P, "psmma_" + kind)
    return compute(rows, k, alpha, A_panel, gen, beta, Q_panel, **kw)
