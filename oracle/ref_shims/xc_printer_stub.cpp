// Link stub for the reference's OBJ mesh builder (geometry/xenocollide/XCPrinter.cpp),
// whose real implementation needs the un-vendored quickhull submodule.  Mesh printing
// is never reached on the Monte Carlo path the oracle drives; calling it throws.
#include <stdexcept>
#include "geometry/xenocollide/XCPrinter.h"

Polyhedron XCPrinter::buildPolyhedron0(const AbstractXCGeometry &, std::size_t) {
    throw std::runtime_error("XCPrinter::buildPolyhedron0 is not available in the oracle build");
}
