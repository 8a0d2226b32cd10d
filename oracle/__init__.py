"""CPU restatement of MCF's SDPD step: test infrastructure (parity checker
and CPU baseline), never part of the product path."""
