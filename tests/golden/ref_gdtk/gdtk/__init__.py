"""The reference's gdtk Python package, reduced to its gas module (copied verbatim by
tests/golden/make_fixtures.sh).  Test infrastructure for the drop-in test of the C ABI."""
