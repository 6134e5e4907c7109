"""ORACLE / TEST INFRASTRUCTURE ONLY: CPU restatement of the reference's pricing path (see oracle.py)."""
