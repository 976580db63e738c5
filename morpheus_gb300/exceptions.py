"""Exception classes with the reference's names
(core/src/Morpheus_Exceptions.hpp:32-73), mapped from C-ABI status codes."""
from __future__ import annotations


class MorpheusException(RuntimeError):
    """Base of all library errors."""


class NotImplementedException(MorpheusException):
    pass


class FormatConversionException(MorpheusException):
    pass


class InvalidInputException(MorpheusException):
    pass


class RuntimeException(MorpheusException):
    pass


class IOException(MorpheusException):
    pass


class CudaException(RuntimeException):
    """A CUDA runtime call inside the library failed."""


class TimeoutException(RuntimeException):
    """A bounded device-side wait ran out."""


class BadArgumentException(InvalidInputException):
    """Null pointer, negative size or bad enum passed to the C ABI."""


class AllocationException(RuntimeException):
    """Device allocation failed."""


_BY_STATUS = {
    1: NotImplementedException,
    2: FormatConversionException,
    3: InvalidInputException,
    4: RuntimeException,
    5: IOException,
    6: CudaException,
    7: TimeoutException,
    8: BadArgumentException,
    9: AllocationException,
}


def raise_for_status(status: int, where: str, cuda_text: str = "") -> None:
    cls = _BY_STATUS.get(status, RuntimeException)
    msg = f"{where} failed with status {status}"
    if status in (6, 9) and cuda_text:
        msg += f" ({cuda_text})"
    raise cls(msg)
