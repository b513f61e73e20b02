"""GB300-native collocated finite-volume SIMPLE/PISO step with the API of warp_cfd."""


def set_krylov_path(mode: str = "auto") -> None:
    """Choose the CG kernel: 'auto' (cluster-resident when the system fits one thread-block
    cluster's shared memory, else grid-cooperative), 'grid', 'cluster', or 'cluster1'
    (cluster-resident with the single-reduction arrangement of CG: one cluster all-reduce
    per iteration, the textbook iterates up to rounding)."""
    from . import _lib

    _lib.call("wcfd_set_krylov_path", {"auto": 0, "grid": 1, "cluster": 2, "cluster1": 3}[mode])
