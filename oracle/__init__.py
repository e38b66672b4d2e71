"""CPU restatement of the reference NDT path: test infrastructure only (the checker and the
timed CPU baseline). The product never imports this package."""
