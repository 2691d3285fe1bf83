"""Argument and ordering errors of the Python API that need no GPU: the
CycleBuilder call order (GMG/CycleBuilder.h:97-192, test/GMG/CycleBuilder_MPI1.cpp:56-309)
and unknown cycle types."""
import pytest

from thunderegg_gb300 import CycleBuilder, CycleOpts
from thunderegg_gb300.capi import TE_ERR_INVALID, TE_ERR_UNSUPPORTED, TeError


def test_cycle_builder_order():
    op, sm, r, i = object(), object(), object(), object()
    b = CycleBuilder(CycleOpts())
    with pytest.raises(TeError) as e:
        b.addIntermediateLevel(op, sm, r, i)  # before the finest level
    assert e.value.code == TE_ERR_INVALID
    with pytest.raises(TeError):
        b.addCoarsestLevel(op, sm, i)  # before the finest level
    with pytest.raises(TeError):
        b.getCycle()  # no coarsest level
    b.addFinestLevel(op, sm, r)
    with pytest.raises(TeError):
        b.addFinestLevel(op, sm, r)  # twice
    b.addIntermediateLevel(op, sm, r, i)
    b.addCoarsestLevel(op, sm, i)
    with pytest.raises(TeError):
        b.addIntermediateLevel(op, sm, r, i)  # after the coarsest level
    with pytest.raises(TeError):
        b.addCoarsestLevel(op, sm, i)  # twice


def test_unknown_cycle_type():
    op, sm, r, i = object(), object(), object(), object()
    b = CycleBuilder(CycleOpts(cycle_type="X"))
    b.addFinestLevel(op, sm, r)
    b.addCoarsestLevel(op, sm, i)
    with pytest.raises(TeError) as e:
        b.getCycle()
    assert e.value.code == TE_ERR_UNSUPPORTED
