"""INI configuration with evaluated values, as in ``pyprop/Config.py``.

Every option value is a Python expression evaluated in the project namespace
(``pyprop/Config.py:21-30``); ``base = "Other"`` imports another section first
(``:13-19``); ``[Import] files = [...]`` pulls in further INI files (``:86-120``);
``%(name)s`` interpolation works as in ConfigParser. Sections hand themselves to objects
through ``Apply`` -> ``ApplyConfigSection`` (``:43-46``), the whole config through
``ApplyConfig`` (``:63-66``).
"""
from __future__ import annotations

import configparser
import io
import logging
import math
import os

import numpy

ProjectNamespace: dict = {}
"""Names visible to option expressions (the reference's ``ProjectNamespace``).

The package registers its propagators, solvers, potentials and time functions here;
user scripts add their own (``ProjectNamespace.update(globals())``)."""

_BASE_NAMES = {name: getattr(numpy, name) for name in
               ("pi", "sin", "cos", "exp", "sqrt", "log", "array", "arange", "linspace", "zeros", "ones", "r_")}
_BASE_NAMES.update({"math": math, "numpy": numpy, "None": None, "True": True, "False": False})

_log = logging.getLogger("pyprop_gb300.config")


class Section:
    """One config section; option names become attributes."""

    def __init__(self, name, cfg=None):
        self.name = name
        if cfg is not None:
            self.LoadConfig(name, cfg)

    def LoadConfig(self, name, cfg):
        for option in cfg.options(name):
            if option == "base":
                self.LoadConfig(eval(cfg.get(name, option)), cfg)
            else:
                self.SetOptionString(option, cfg.get(name, option))

    def SetOptionString(self, option, text):
        glob = dict(_BASE_NAMES)
        glob.update(ProjectNamespace)
        try:
            value = eval(text, glob, self.__dict__)
        except Exception as exc:  # the reference logs and skips unknown names
            _log.error("Could not evaluate %s.%s = %s (%s)", self.name, option, text, exc)
            return
        self.Set(option, value)

    def Set(self, option, value):
        if option in ("name", "SetOptionString", "Set", "Get"):
            raise ValueError("Invalid option name %s" % option)
        self.__dict__[option] = value

    def Get(self, option):
        return self.__dict__[option]

    def get(self, option, default=None):
        return self.__dict__.get(option, default)

    def Exists(self, option):
        return option in self.__dict__

    def Apply(self, other):
        if hasattr(other, "ApplyConfigSection"):
            other.ApplyConfigSection(self)

    def __repr__(self):
        items = {k: v for k, v in self.__dict__.items() if k not in ("Config",)}
        return "Section(%s)" % items


class Config:
    """All sections of a parsed config (``pyprop/Config.py:48-84``)."""

    def __init__(self, cfg):
        self.cfgObj = cfg
        for sname in cfg.sections():
            if sname == "GetSection":
                raise ValueError("Invalid section name %s" % sname)
            sec = Section(sname, cfg)
            sec.Config = self
            self.__dict__[sname] = sec

    def GetSection(self, name):
        return self.__dict__[name]

    def Apply(self, other):
        if hasattr(other, "ApplyConfig"):
            other.ApplyConfig(self)

    def SetValue(self, section, option, value):
        """Set ``section.option`` to ``value`` in both the parsed and the raw config."""
        self.cfgObj.set(section, option, repr(value))
        self.__dict__[section].Set(option, value)


def _parser():
    return configparser.ConfigParser(interpolation=configparser.BasicInterpolation())


def Load(fileName):
    """Parse an INI file (following ``[Import] files``) into a :class:`Config`."""
    files = []
    pending = [(".", fileName)]
    while pending:
        cur_dir, cur_file = pending.pop()
        path = os.path.abspath(os.path.expanduser(os.path.expandvars(os.path.join(cur_dir, cur_file))))
        files.insert(0, path)
        cfg = _parser()
        with open(path) as fh:
            cfg.read_file(fh)
        if cfg.has_section("Import") and cfg.has_option("Import", "files"):
            for f in eval(cfg.get("Import", "files")):
                pending.insert(0, (os.path.dirname(path), f))
    cfg = _parser()
    for path in files:
        with open(path) as fh:
            cfg.read_file(fh)
    return Config(cfg)


def LoadString(text):
    """Parse INI text into a :class:`Config` (no ``[Import]`` support)."""
    cfg = _parser()
    cfg.read_file(io.StringIO(text))
    return Config(cfg)


def UpdateConfig(conf, updateParams):
    """Return a new config with ``[(section, option, value), ...]`` applied
    (``pyprop/Config.py:123-158``)."""
    tmp = Config(conf.cfgObj)
    for section, option, value in updateParams:
        if not tmp.cfgObj.has_section(section):
            tmp.cfgObj.add_section(section)
        tmp.cfgObj.set(section, option, repr(value))
    return Config(tmp.cfgObj)
