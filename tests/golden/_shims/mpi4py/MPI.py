"""Single-rank stand-in for ``mpi4py.MPI``: every collective on one rank is an
identity or a copy.  Test infrastructure only (golden-fixture generation)."""
import numpy as _np


class _Op:
    def __init__(self, name):
        self.name = name


SUM, MAX, MIN, PROD, LAND, LOR = (_Op(n) for n in ("SUM", "MAX", "MIN", "PROD", "LAND", "LOR"))
IN_PLACE = object()
COMM_TYPE_SHARED = 1


class Datatype:
    def __init__(self, name):
        self.name = name


INT, LONG, FLOAT, DOUBLE, COMPLEX, DOUBLE_COMPLEX = (
    Datatype(n) for n in ("INT", "LONG", "FLOAT", "DOUBLE", "COMPLEX", "DOUBLE_COMPLEX")
)
Op = _Op


def _arr(buf):
    """Return the array part of an mpi4py-style buffer spec."""
    if isinstance(buf, (list, tuple)):
        return buf[0]
    return buf


def _copy(src, dst):
    s = _arr(src)
    d = _arr(dst)
    if s is IN_PLACE or s is d:
        return
    try:
        d[...] = s
    except TypeError:  # torch tensor
        d.copy_(s)


class Request:
    def Wait(self):
        return None

    def wait(self):
        return None

    def Test(self):
        return True


class _Group:
    def Incl(self, *a, **k):
        return self

    def Excl(self, *a, **k):
        return self


class Comm:
    rank = 0
    size = 1

    def Get_rank(self):
        return 0

    def Get_size(self):
        return 1

    def Split_type(self, *a, **k):
        return self

    def Split(self, *a, **k):
        return self

    def Create_cart(self, *a, **k):
        return self

    def Sub(self, *a, **k):
        return self

    def Dup(self):
        return self

    def Create_group(self, *a, **k):
        return self

    def Get_group(self):
        return _Group()

    def Free(self):
        pass

    def Barrier(self):
        pass

    barrier = Barrier

    def allreduce(self, x, op=SUM):
        return x

    def bcast(self, x, root=0):
        return x

    def allgather(self, x):
        return [x]

    def gather(self, x, root=0):
        return [x]

    def scatter(self, x, root=0):
        return x[0]

    def Bcast(self, buf, root=0):
        pass

    def Allreduce(self, sendbuf, recvbuf, op=SUM):
        _copy(sendbuf, recvbuf)

    def Reduce(self, sendbuf, recvbuf, op=SUM, root=0):
        _copy(sendbuf, recvbuf)

    def Iallreduce(self, sendbuf, recvbuf, op=SUM):
        _copy(sendbuf, recvbuf)
        return Request()

    def Allgather(self, sendbuf, recvbuf):
        _copy(sendbuf, recvbuf)

    def Allgatherv(self, sendbuf, recvbuf):
        _copy(sendbuf, recvbuf)

    def Alltoallv(self, sendbuf, recvbuf):
        _copy(sendbuf, recvbuf)

    def Ialltoallv(self, sendbuf, recvbuf):
        _copy(sendbuf, recvbuf)
        return Request()

    def Ibcast(self, buf, root=0):
        return Request()


COMM_WORLD = Comm()
COMM_SELF = COMM_WORLD
COMM_NULL = None


def Get_library_version():
    return "single-rank stand-in"


def Wtime():
    import time

    return time.time()


_ = _np
