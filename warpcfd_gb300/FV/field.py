class Field:
    """Named field with its column in ``cell_values`` (warp_cfd/FV/field.py:1-4)."""

    def __init__(self, name, index=-1):
        self.name = name
        self.index = index
