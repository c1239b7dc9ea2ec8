class DataFrame:
    def __init__(self, *a, **k): raise RuntimeError("pandas stub")
class Series(DataFrame): pass
