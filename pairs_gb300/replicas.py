"""Independent replicas on several GPUs (one process per GPU, torchrun).

The path runs one periodic domain per GPU and does not shard; with N processes each
GPU advances its own replica, and the whole-job throughput is the units all ranks
processed divided by the slowest rank's time.  No collective touches the data path:
the only exchange is this final reduction of two scalars.
"""
import torch


def job_throughput(units_local, ms_local, dist=None, device=None):
    """(units per second over all ranks, max ms over ranks).  `dist` is
    torch.distributed (initialised) or None for a single process."""
    if dist is None or not dist.is_available() or not dist.is_initialized():
        return units_local / (ms_local / 1e3), ms_local
    dev = device if device is not None else torch.device("cpu")
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(units_local)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    ms = float(t.item())
    return float(u.item()) / (ms / 1e3), ms


def init_from_env(os_environ):
    """Initialise torch.distributed from torchrun's environment: NCCL when a GPU is
    present, gloo otherwise.  Returns (dist or None, rank, world, local_rank)."""
    ws = int(os_environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1, 0
    import torch.distributed as dist
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    dist.init_process_group(backend)
    return dist, int(os_environ["RANK"]), ws, int(os_environ.get("LOCAL_RANK", "0"))
