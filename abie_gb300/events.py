"""Event exceptions raised by this package's ctypes binding.

They have the names, fields (t, obj1, obj2, distance) and messages of the
reference's abie/events.py:1-34, so handlers written against those classes
read the same attributes.  They are separate classes: an ``except`` clause
naming ``abie.events.CloseEncounterException`` does not catch this module's
exception.  Code that runs the reference's own Python package on this
library (its unchanged abie/clibabie.py loading libabie_gb300) raises the
reference's classes, since that binding turns the return codes 1 / 2 into
its own exceptions.
"""


class ParticleException(Exception):
    """A two-body event at time t between obj1 and obj2 at a distance."""

    def __init__(self, t, obj1, obj2, distance):
        super().__init__(t, obj1, obj2, distance)
        self.t = t
        self.obj1 = obj1
        self.obj2 = obj2
        self.distance = distance


class CloseEncounterException(ParticleException):
    def __str__(self):
        return ("Close encounter detected between particle #%d and particle #%d with a "
                "distance of %g at t = %g" % (self.obj1, self.obj2, self.distance, self.t))


class CollisionException(ParticleException):
    def __str__(self):
        return ("Collision detected between particle #%d and particle #%d with a "
                "distance of %g at t = %g" % (self.obj1, self.obj2, self.distance, self.t))


class AbieError(RuntimeError):
    """A negative return code of libabie_gb300 (device, capacity, timeout...)."""

    def __init__(self, code, message):
        super().__init__("libabie_gb300 error %d: %s" % (code, message))
        self.code = code
