"""
Attribute-bag parameter classes with the shape of the reference's
helpers.parameters (src/helpers/parameters.py:7-112): `Parameters` holds
public attributes, `check()` lists the unset ones, and both print as an
indented tree.
"""
from __future__ import annotations


class TreePrintable(object):
    """Prints the class name followed by its public attributes and
    properties, one per indented line, nesting TreePrintable values
    (src/helpers/parameters.py:7-83)."""

    @property
    def _print_name(self):
        return None

    def __repr__(self, prefix="", level=0, blanks=4):
        name = self.__class__.__name__ if self._print_name is None else self._print_name
        name = (" " * (level * blanks)) + prefix + name
        items = [(k, v) for k, v in vars(self).items() if not k.startswith("_")]
        for cls in type(self).mro()[::-1]:
            for pname, thing in cls.__dict__.items():
                if isinstance(thing, property) and not pname.startswith("_"):
                    try:
                        value = thing.__get__(self)
                    except AttributeError:
                        value = "[no getter defined]"
                    items.append(("[property] %s" % pname, value))
        items.sort(key=lambda kv: kv[0].lower())
        lines = []
        for k, v in items:
            if isinstance(v, TreePrintable):
                lines.append(v.__repr__(prefix="%s: " % k, level=level + 1, blanks=blanks))
            else:
                lines.append((" " * ((level + 1) * blanks)) + "%s: %s" % (k, v))
        if not lines:
            lines = [(" " * ((level + 1) * blanks)) + "[no attributes]"]
        return name + "\n" + "\n".join(lines)


class Parameters(TreePrintable):
    """Parameters as instance attributes (src/helpers/parameters.py:86-112)."""

    def check(self, raise_e=False):
        """Names of the parameters still None; raise RuntimeError instead
        when raise_e is True."""
        unset = sorted(str(k) for k, v in vars(self).items() if v is None)
        if unset:
            msg = "The following parameters have not been set:\n" + "\n".join(unset)
            if raise_e:
                raise RuntimeError(msg)
            print(msg)
            return unset
        return None
