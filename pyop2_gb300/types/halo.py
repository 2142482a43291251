"""Halo (pyop2/types/halo.py:4-58): the abstract description of which Set
entries a rank sends and receives.  A single-process run has no halos to
exchange, so nothing here implements one; the base class is kept so that
user code subclassing or checking against it keeps working."""
import abc


class Halo(abc.ABC):

    @property
    @abc.abstractmethod
    def comm(self):
        """The communicator of the halo exchange."""

    @property
    @abc.abstractmethod
    def local_to_global_numbering(self):
        """The global numbers of the local entries."""

    @abc.abstractmethod
    def global_to_local_begin(self, dat, insert_mode):
        """Start copying owned values into the halo entries of `dat`."""

    @abc.abstractmethod
    def global_to_local_end(self, dat, insert_mode):
        """Finish copying owned values into the halo entries of `dat`."""

    @abc.abstractmethod
    def local_to_global_begin(self, dat, insert_mode):
        """Start sending halo contributions of `dat` to their owners."""

    @abc.abstractmethod
    def local_to_global_end(self, dat, insert_mode):
        """Finish sending halo contributions of `dat` to their owners."""
