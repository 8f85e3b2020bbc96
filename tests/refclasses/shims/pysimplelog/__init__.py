"""Minimal stand-in for the third-party logger package ``pysimplelog``
(>= 2.0.0), which fullrmc imports in ``Globals.py:25`` and which is not
installed here.  Written from fullrmc's own use of it (``Globals.py:72-150``
and the ``LOGGER.<level>(message)`` call sites): a logger class that fullrmc
subclasses, with log types added by name, and level methods that return
something ``assert cond, LOGGER.error(...)`` and ``raise LOGGER.error(...)``
can use.  Nothing is printed or written: test infrastructure only.
"""


class LoggedError(Exception):
    """What ``error`` and ``critical`` return: an exception carrying the message."""


class SingleLogger(object):
    def __init__(self, name="logger", *args, **kwargs):
        self.name = name
        self.log_types = {}
        self.minimum_level = 0
        self.custom_init()

    def custom_init(self):
        pass

    def set_log_file_basename(self, *args, **kwargs):
        pass

    def add_log_type(self, logType, name=None, level=0, *args, **kwargs):
        self.log_types[logType] = (name, level)

    def set_minimum_level(self, level=0, *args, **kwargs):
        self.minimum_level = level

    def force_log_type_flags(self, *args, **kwargs):
        pass

    def log(self, logType, message, *args, **kwargs):
        return message

    def debug(self, message, *args, **kwargs):
        return message

    def info(self, message, *args, **kwargs):
        return message

    def warn(self, message, *args, **kwargs):
        return message

    warning = warn

    def error(self, message, *args, **kwargs):
        return LoggedError(message)

    def critical(self, message, *args, **kwargs):
        return LoggedError(message)
