// Library-wide C-ABI helpers.
#include "snapgb300.h"

extern "C" int sg_version(void) { return 100; }

extern "C" const char* sg_status_string(int status) {
  switch (status) {
    case SG_OK: return "ok";
    case SG_ERR_ARG: return "invalid argument";
    case SG_ERR_RANGE: return "position out of range of the genome or chromosome";
    case SG_ERR_CAP: return "buffer too small";
    case SG_ERR_CUDA: return "CUDA error";
    case SG_ERR_NUMERIC: return "numerical breakdown";
    case SG_ERR_TIMEOUT: return "device-side wait timed out";
    case SG_ERR_PARSE: return "malformed fragment record";
    case SG_ERR_UNSORTED: return "Please sort fragment file by barcodes";
    case SG_ERR_CONVERT: return "fragment size does not fit the matrix value type";
    case SG_ERR_COLLISION: return "barcode hash collision";
    default: return "unknown status";
  }
}
