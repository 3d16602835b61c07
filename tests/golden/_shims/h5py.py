"""Stand-in for h5py (not installed where golden fixtures are generated).
Opening a file always fails, so checkpoints are never read or written."""


class File:
    def __init__(self, *a, **k):
        raise OSError("h5py stand-in: HDF5 files are unavailable")


class Dataset:
    pass


class Group:
    pass
