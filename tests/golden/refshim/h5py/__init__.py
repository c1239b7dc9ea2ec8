class File:  # stub
    def __init__(self, *a, **k):
        raise RuntimeError("h5py stub")
class Dataset: pass
class Group: pass
