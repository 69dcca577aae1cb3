"""A minimal i-PI server (the side the fnet socket client talks to): sends positions, asks for
forces, and records what the client returns.  Test infrastructure for the socket client."""

from __future__ import annotations

import os
import socket
import struct

import numpy as np

MSGLEN = 12


def _hdr(s):
    return s.encode().ljust(MSGLEN, b" ")


class IpiServer:
    """Listens on 127.0.0.1 (port chosen by the OS) or on a UNIX socket path."""

    def __init__(self, unix_path=None):
        if unix_path:
            if os.path.exists(unix_path):
                os.unlink(unix_path)
            self.srv = socket.socket(socket.AF_UNIX, socket.SOCK_STREAM)
            self.srv.bind(unix_path)
            self.port = 0
        else:
            self.srv = socket.socket(socket.AF_INET, socket.SOCK_STREAM)
            self.srv.bind(("127.0.0.1", 0))
            self.port = self.srv.getsockname()[1]
        self.srv.listen(1)
        self.srv.settimeout(120.0)
        self.conn = None

    def accept(self):
        self.conn, _ = self.srv.accept()
        self.conn.settimeout(120.0)

    def _recv(self, n):
        buf = b""
        while len(buf) < n:
            chunk = self.conn.recv(n - len(buf))
            if not chunk:
                raise ConnectionError("client closed the connection")
            buf += chunk
        return buf

    def _status(self):
        self.conn.sendall(_hdr("STATUS"))
        return self._recv(MSGLEN).decode().strip()

    def evaluate(self, pos, h, statuses=2):
        """One i-PI force evaluation: pos [n, 3] Bohr, h [3, 3] with the lattice vectors as
        columns.  Returns (energy, forces [n, 3], virial [3, 3] as sent, extra string)."""
        for _ in range(statuses):
            assert self._status() == "READY"
        self.conn.sendall(_hdr("POSDATA"))
        self.conn.sendall(np.ascontiguousarray(h, dtype="<f8").tobytes())  # row-major h
        self.conn.sendall(np.ascontiguousarray(np.linalg.inv(h), dtype="<f8").tobytes())
        self.conn.sendall(struct.pack("<i", len(pos)))
        self.conn.sendall(np.ascontiguousarray(pos, dtype="<f8").tobytes())
        for _ in range(statuses):
            assert self._status() == "HAVEDATA"
        self.conn.sendall(_hdr("GETFORCE"))
        assert self._recv(MSGLEN).decode().strip() == "FORCEREADY"
        e = struct.unpack("<d", self._recv(8))[0]
        n = struct.unpack("<i", self._recv(4))[0]
        f = np.frombuffer(self._recv(24 * n), dtype="<f8").reshape(n, 3)
        vir = np.frombuffer(self._recv(72), dtype="<f8").reshape(3, 3)
        nextra = struct.unpack("<i", self._recv(4))[0]
        extra = self._recv(nextra).decode() if nextra else ""
        return e, f, vir, extra

    def exit(self):
        self._status()
        self.conn.sendall(_hdr("EXIT"))

    def close(self):
        if self.conn:
            self.conn.close()
        self.srv.close()
