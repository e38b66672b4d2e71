"""CPU restatement of the reference NDT path: test infrastructure only (the oracle and the
timed CPU baseline). The product never imports this package."""
