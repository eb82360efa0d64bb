"""CPU oracle (test infrastructure only): numpy restatement of the reference path."""
