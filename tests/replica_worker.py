"""Worker for the two-rank replica tests (a module of its own so spawned processes can import it)."""
import os


def whole_job_rate_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from spi_gb300 import replicas
    r = replicas.init("gloo")
    r.barrier()
    local_ms = 100.0 * (rank + 1)              # rank 1 is the slower replica
    value, ms = r.whole_job_rate(1000.0, local_ms)
    out[rank] = (value, ms, r.rank, r.world)
    r.close()
