"""Test oracle (CPU restatement of the MTGP reference).  TEST ONLY."""
