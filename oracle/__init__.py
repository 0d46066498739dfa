"""CPU oracle of stardust-gb300 -- test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU legs; the
product library never loads it.
"""
