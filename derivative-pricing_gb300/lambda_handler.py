"""AWS Lambda entry point over the GPU engine, for the reference's demo API
(infra/lambda/handler.py, request.py, cfa_invariants.py): an API Gateway HTTP API
(Lambda proxy integration, payload format 2.0) with two routes,

    GET  /cfa-invariants   {"invariants": [{"module", "invariant", "pass", "deviation"}, ...]}
    POST /price            one JSON request object -> one JSON result object

and the same status codes: 400 with {"error": message} for a malformed body or
request, 404 for an unknown route, 500 for anything unexpected.  The request schema
is the JSON CLI's (same products, request kinds and fields) in the Lambda layer's
dialect: its validation messages, the path-count cap (MAX_PATH_COUNT, 5,000,000 as
the reference's; the environment variable MCD_MAX_PATH_COUNT overrides it), binomial
steps in 1..20,000 and the "antithetic"/"control_variate" toggles.  Each request is
handled in process by the shim library's request handler (request.cpp), which prices
on the GPU; nothing here prices on the CPU except the closed forms.

Deployed in place of the reference's three files, with this directory, the built
libraries under build/ and a GPU on the host.
"""
from __future__ import annotations

import ctypes as C
import json
import os

PKG = os.path.dirname(os.path.abspath(__file__))
SHIM_PATH = os.path.join(PKG, "build", "libmcd_shim.so")
MAX_PATH_COUNT = int(os.environ.get("MCD_MAX_PATH_COUNT", "5000000"))
DIALECT_LAMBDA = 1
OK, REQUEST_ERROR, INTERNAL_ERROR = 0, 1, 2

_HEADERS = {"Content-Type": "application/json"}
_shim = None


class RequestError(Exception):
    """A malformed or out-of-bounds request: answered with 400."""


def _lib():
    global _shim
    if _shim is None:
        if not os.path.exists(SHIM_PATH):
            raise RuntimeError(f"{SHIM_PATH} not found: build it with derivative-pricing_gb300/build.py")
        lib = C.CDLL(SHIM_PATH)
        lib.mcd_shim_handle_request.restype = C.c_void_p
        lib.mcd_shim_handle_request.argtypes = [C.c_char_p, C.c_int, C.c_uint64, C.POINTER(C.c_int)]
        lib.mcd_shim_free.restype = None
        lib.mcd_shim_free.argtypes = [C.c_void_p]
        _shim = lib
    return _shim


def handle_request(req):
    """One request object -> its result object (raises RequestError)."""
    if not isinstance(req, dict):
        raise RequestError("request body must be a JSON object")
    lib = _lib()
    status = C.c_int(INTERNAL_ERROR)
    ptr = lib.mcd_shim_handle_request(json.dumps(req).encode(), DIALECT_LAMBDA, MAX_PATH_COUNT, C.byref(status))
    if not ptr:
        raise RuntimeError("out of memory")
    try:
        body = json.loads(C.string_at(ptr).decode())
    finally:
        lib.mcd_shim_free(ptr)
    if status.value == REQUEST_ERROR:
        raise RequestError(body["error"])
    if status.value != OK:
        raise RuntimeError(body["error"])
    return body


def cfa_invariant_table():
    """The no-arbitrage invariants of the closed forms, as the demo's table rows."""
    from report import cfa_invariants
    return [{"module": m, "invariant": name, "pass": bool(ok), "deviation": dev}
            for m, name, ok, dev in cfa_invariants()]


def _response(status_code, body):
    return {"statusCode": status_code, "headers": dict(_HEADERS), "body": json.dumps(body)}


def lambda_handler(event, _context):
    route = event.get("routeKey", "")
    try:
        if route == "GET /cfa-invariants":
            return _response(200, {"invariants": cfa_invariant_table()})
        if route == "POST /price":
            try:
                req = json.loads(event.get("body") or "{}")
            except json.JSONDecodeError as e:
                return _response(400, {"error": f"malformed JSON body: {e}"})
            try:
                return _response(200, handle_request(req))
            except RequestError as e:
                return _response(400, {"error": str(e)})
        return _response(404, {"error": f"no route for '{route}'"})
    except Exception as e:  # noqa: BLE001 -- a clean JSON 500, never an opaque gateway error
        return _response(500, {"error": f"internal error: {e}"})
