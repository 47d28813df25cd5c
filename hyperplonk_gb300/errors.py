"""BackendError kinds of the reference (backend/src/errors.rs:16-21) and the
ABI status mapping of backend/src/ascend910b3/status.rs."""


class BackendError(Exception):
    """Base class of backend failures."""


class InvalidParameters(BackendError):
    """Invalid parameters (malformed shapes, non-canonical values, zero denominators)."""


class InvalidState(BackendError):
    """Invalid execution state (round misuse, exhausted or poisoned state, device failure)."""


STATUS_SUCCESS = 0
STATUS_INVALID_PARAMETERS = 1
STATUS_INVALID_STATE = 2
STATUS_NOT_IMPLEMENTED = 3


def check_status(status, operation: str) -> None:
    """status.rs:into_result: only (0, 0) succeeds; kind 1 keeps its category,
    every other kind is InvalidState."""
    kind, code = status.kind, status.native_code
    if kind == STATUS_SUCCESS and code == 0:
        return
    if kind == STATUS_INVALID_PARAMETERS:
        raise InvalidParameters(f"{operation} failed (kind={kind}, native_code={code})")
    if kind == STATUS_NOT_IMPLEMENTED:
        raise InvalidState(f"{operation} not implemented (kind=3, native_code={code})")
    raise InvalidState(f"{operation} failed (kind={kind}, native_code={code})")
