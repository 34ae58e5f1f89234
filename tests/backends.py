"""Uniform construction interface over the oracle and the product library for the ported tests."""
import pytest


def make_tree(backend, size, dim):
    if backend == "oracle":
        from oracle import oracle
        return oracle.Tree(size, dim)
    import shocovox_gb300 as svo
    return svo.Octree(size, dim)


def creation_error(backend, size, dim):
    if backend == "oracle":
        from oracle import oracle
        try:
            oracle.Tree(size, dim)
        except oracle.OracleError as e:
            return e.code
        return 0
    import shocovox_gb300 as svo
    try:
        svo.Octree(size, dim)
    except svo.OctreeError as e:
        return e.code
    return 0
