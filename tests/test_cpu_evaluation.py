"""Host-side checks of the diagnostics drop-ins (lacmopy_gb300/evaluation.py)
that need no GPU: the reference's particle-ID convention is enforced."""
import numpy as np
import pytest


def test_id_list_must_be_the_reference_order():
    from lacmopy_gb300.evaluation import _check_ids
    _check_ids(np.arange(5), 5)
    _check_ids(None, 5)
    with pytest.raises(ValueError):
        _check_ids(np.array([1, 0, 2, 3, 4]), 5)
