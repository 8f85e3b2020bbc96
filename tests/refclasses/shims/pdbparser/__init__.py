"""Minimal stand-in for the third-party package ``pdbparser`` (>= 0.1.8),
which fullrmc's constraint modules import and which is not installed here.
Only the three functions those modules call are provided (see
``Utilities``); test infrastructure only."""
