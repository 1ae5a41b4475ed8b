// sed_handles.cuh -- the opaque handles of the C ABI (include/sed_capi.h).
//
// Each handle holds a shared reference to its implementation object, so an
// operator keeps its sector, catalog and group alive and destroy order is
// free.  Every translation unit that dereferences a handle includes this one
// definition.
#pragma once

#include <memory>

#include "../../include/sed_capi.h"
#include "sed_internal.cuh"

namespace sed {
struct BatchImpl;
}

struct sed_group {
  std::shared_ptr<sed::GroupImpl> p;
};
struct sed_catalog {
  std::shared_ptr<sed::CatalogImpl> p;
};
struct sed_sector {
  std::shared_ptr<sed::SectorImpl> p;
};
struct sed_op {
  std::shared_ptr<sed::OpImpl> p;
};
struct sed_batch {
  std::shared_ptr<sed::BatchImpl> p;
};
