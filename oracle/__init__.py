"""ORACLE — test infrastructure, not product code.

CPU restatements of the reference's hot path (and of the engine's counter-
based noise streams) that the tests, the smoke check and the bench's CPU
baseline compare the GPU engine against.  The product path never imports
this package."""
