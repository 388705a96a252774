"""CPU build of the reference's own sources (TEST INFRASTRUCTURE; see build_ref.py)."""
