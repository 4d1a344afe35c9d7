"""ORACLE (test infrastructure only): pre-builds the C restatement (the sequential
reduction library) so the first checker or baseline run does not pay for it."""


def build():
    from . import cref
    cref._reducer()
