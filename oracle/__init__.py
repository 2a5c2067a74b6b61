"""ORACLE — test infrastructure only: the CPU restatement of PeleC's MOL
right-hand side used as the checker and as the timed CPU baseline.  Never
imported by the product (pelec_gb300)."""
