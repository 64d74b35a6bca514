"""CPU oracle of the RHF-CCSD path (test infrastructure only; see ``oracle/ccsd.py``)."""
