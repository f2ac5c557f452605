"""CPU FP64 oracle of the eff_pot hot path: test infrastructure only (the
parity checker and the timed CPU baseline).  The product never imports it."""
