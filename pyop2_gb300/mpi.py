"""Communicators of a single-process, single-GPU run.

The reference runs one MPI rank per process and exports its ``mpi`` module
as ``op2.MPI`` (pyop2/mpi.py: ``COMM_WORLD``, ``COMM_SELF``, the
``collective`` decorator, ``internal_comm``).  Here every process is one
rank (several GPUs are independent replicas), so the communicators are
stand-ins with rank 0 and size 1 whose collectives return their input: user
code that passes ``comm=op2.MPI.COMM_WORLD`` or reduces a local value over
it runs unchanged.
"""
import functools

__all__ = ["COMM_WORLD", "COMM_SELF", "SingleProcessComm", "collective", "internal_comm",
           "is_pyop2_comm", "PyOP2CommError"]


class PyOP2CommError(ValueError):
    pass


class SingleProcessComm:
    """The parts of an mpi4py intracommunicator user code touches, for one
    rank: rank/size queries, barrier, broadcast, (all)reduce, (all)gather."""

    def __init__(self, name):
        self.name = name

    rank = property(lambda self: 0)
    size = property(lambda self: 1)

    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def Get_name(self):
        return self.name

    def Set_name(self, name):
        self.name = name

    def barrier(self):
        return None

    Barrier = barrier

    def bcast(self, obj, root=0):
        return obj

    def allreduce(self, obj, op=None):
        return obj

    def reduce(self, obj, op=None, root=0):
        return obj

    def allgather(self, obj):
        return [obj]

    def gather(self, obj, root=0):
        return [obj]

    def Dup(self):
        return SingleProcessComm(self.name)

    def Free(self):
        return None

    def __repr__(self):
        return "SingleProcessComm(%r)" % self.name


COMM_WORLD = SingleProcessComm("PYOP2_COMM_WORLD")
COMM_SELF = SingleProcessComm("PYOP2_COMM_SELF")


def is_pyop2_comm(comm):
    return isinstance(comm, SingleProcessComm)


def internal_comm(comm, obj=None):
    """The communicator PyOP2 objects use internally for `comm` (itself
    here: there is no duplication to track on one rank)."""
    if comm is None:
        return COMM_WORLD
    return comm


def collective(fn):
    """Marks a call all ranks must make (pyop2/mpi.py:164-221); on one rank
    it changes nothing."""
    @functools.wraps(fn)
    def wrapper(*args, **kwargs):
        return fn(*args, **kwargs)
    wrapper.__collective__ = True
    return wrapper
