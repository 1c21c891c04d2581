// No-op definitions of the reference's NetCDF writers (include/io/netCDF_writer.hpp,
// include/io/sanity_checks_netdcdf_writer.hpp), for builds of the reference's own code
// on machines without libnetcdf-c++4.  Test infrastructure only.
#include "include/io/netCDF_writer.hpp"
#include "include/io/sanity_checks_netdcdf_writer.hpp"

NetCDFWriter::NetCDFWriter(const std::string &, const Grid &grid, const std::string &,
                           const std::string &, const std::string &, const std::string &, int)
    : grid_(grid), nx_(0), ny_(0) {}
void NetCDFWriter::write_snapshot(const State &, double, double, const std::string &,
                                  const std::string &, const std::string &, const std::string &,
                                  const std::string &, const std::string &) {}
void NetCDFWriter::write_bathymetry(const Array2D &) {}
SanityCheckNetCDFWriter::SanityCheckNetCDFWriter(const std::string &, const std::string &,
                                                 const std::string &, int, double,
                                                 const std::string &, const std::string &,
                                                 const std::string &, const std::string &,
                                                 const std::string &, const std::string &) {}
void SanityCheckNetCDFWriter::write(std::size_t, double, double, double) {}
