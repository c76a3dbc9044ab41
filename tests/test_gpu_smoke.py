"""The entry point's smoke check (one small SKL run on the GPU against the oracle) runs here
too, so that it is exercised with every GPU test pass."""
import pytest

pytestmark = pytest.mark.gpu


def test_entry_smoke(g4s):
    import __graft_entry__ as entry
    entry.smoke()
