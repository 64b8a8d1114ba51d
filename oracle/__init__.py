"""Oracle package (test infrastructure only): the patched-reference build recipe and the
CPU FP64 restatement of the PFDD TDGL hot path.  Imported by tests/, by the smoke check
and by bench.py's CPU-baseline legs; never by the product package."""
