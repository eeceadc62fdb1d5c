"""Shared set-up of the sanitizer builds the tests make (test infrastructure):
gcc's undefined-behaviour checks always, and its address checks when the
address runtime is installed (it must be preloaded into the Python process
that loads a checked library; reports abort)."""
import os
import subprocess


def asan_runtime():
    """Path of gcc's address-sanitizer runtime, or None."""
    try:
        p = subprocess.run(["gcc", "-print-file-name=libasan.so"], capture_output=True, text=True,
                           check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return None
    return p if os.path.isabs(p) and os.path.exists(p) else None


def sanitize_flags():
    """(compiler flags, environment for the child process, the checks' names)."""
    rt = asan_runtime()
    if rt:
        return (["-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined"],
                {"LD_PRELOAD": rt, "ASAN_OPTIONS": "detect_leaks=0", "UBSAN_OPTIONS": "print_stacktrace=1"},
                "address+undefined")
    return (["-fsanitize=undefined", "-fno-sanitize-recover=undefined"], {"UBSAN_OPTIONS": "print_stacktrace=1"},
            "undefined")


def report_found(out: str) -> bool:
    return "runtime error" in out or "ERROR: AddressSanitizer" in out
