// Receiver files in the USGS text format and the grid's geographic mapping (host
// code, no device work).
//
// The format is the one TimeSeries::write_usgs_format writes
// (src/TimeSeries.C:924-1056): a 13-line (for three components) '#' header with the
// station, its requested and recording locations in degrees and the distance between
// them, then one line per record row, the time as %e and every value as %24.17e.
// The header's fixed fields (author, scenario, the placeholder bandwidth 1.234) and
// its column labels, misspellings included, are reproduced as written there so that
// files compare byte for byte with the reference's.
//
// Rotation to geographic components (xyz = 0, src/TimeSeries.C:226-246 and
// :1036-1046): with a the grid azimuth, (ca, sa) = (cos a, sin a), phi the latitude of
// the requested location and D = (x sa + y ca) / (cos phi * meters per degree) in
// radians, the unit north vector in grid components is (tx, ty) normalised from
//   tx = sa + D sin(phi) ca,  ty = ca - D sin(phi) sa,
// and a row (u0, u1, u2) is written as east-west sa u0 + ca u1, north-south
// ty u0 - tx u1 and up-down -u2.
#include <cmath>
#include <cstdio>

#include "../../include/sw4g.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

// values per row of a record mode (SW4G_REC_*), 0 for an unknown mode
int mode_values(int mode)
{
   switch (mode) {
   case SW4G_REC_DISPLACEMENT:
   case SW4G_REC_CURL:
   case SW4G_REC_VELOCITY:
      return 3;
   case SW4G_REC_DIV:
      return 1;
   case SW4G_REC_STRAINS:
      return 6;
   case SW4G_REC_GRADIENT:
      return 9;
   default:
      return 0;
   }
}

// the "# Column c: ..." lines of columns 2.. for a mode
void write_column_labels(FILE* f, int mode, int xyz)
{
   static const char* const disp_xyz[3] = {"X displacement (m)", "Y displacement (m)", "Z displacement (m)"};
   static const char* const disp_geo[3] = {"East-west displacement (m)", "North-sourth displacement (m)",
                                           "Up-down displacement (m)"};
   static const char* const velo_xyz[3] = {"X velocity (m/s)", "Y velocity (m/s)", "Z velocity (m/s)"};
   static const char* const velo_geo[3] = {"East-west velocity (m/s)", "Nort-south velocity (m/s)",
                                           "Up-down velocity (m/s)"};
   static const char* const strain[6] = {"xx", "yy", "zz", "xy", "xz", "yz"};
   static const char* const grad[9] = {"dux/dx", "dux/dy", "dux/dz", "duy/dx", "duy/dy",
                                       "duy/dz", "duz/dx", "duz/dy", "duz/dz"};
   switch (mode) {
   case SW4G_REC_DISPLACEMENT:
   case SW4G_REC_VELOCITY: {
      const char* const* l = mode == SW4G_REC_DISPLACEMENT ? (xyz ? disp_xyz : disp_geo)
                                                           : (xyz ? velo_xyz : velo_geo);
      for (int c = 0; c < 3; c++) std::fprintf(f, "# Column %d: %s\n", c + 2, l[c]);
      break;
   }
   case SW4G_REC_DIV:
      std::fprintf(f, "# Column 2: divergence of displacement ()\n");
      break;
   case SW4G_REC_CURL:
      for (int c = 0; c < 3; c++) std::fprintf(f, "# Column %d: curl of displacement, component %d ()\n", c + 2, c + 1);
      break;
   case SW4G_REC_STRAINS:
      for (int c = 0; c < 6; c++) std::fprintf(f, "# Column %d: %s strain component ()\n", c + 2, strain[c]);
      break;
   case SW4G_REC_GRADIENT:
      // columns 2-9 carry a space before the colon, column 10 none
      for (int c = 0; c < 9; c++)
         std::fprintf(f, c < 8 ? "# Column %d : %s component ()\n" : "# Column %d: %s component ()\n", c + 2,
                      grad[c]);
      break;
   default:
      break;
   }
}

}  // namespace

extern "C" int sw4g_geo_default(sw4g_geo* geo)
{
   if (!geo) return SW4G_BAD_ARGUMENT;
   geo->lon_origin = -118.0;
   geo->lat_origin = 37.0;
   geo->az = 0.0;
   geo->meters_per_degree = 111319.5;
   geo->meters_per_longitude = 87721.0;
   geo->const_meters_per_longitude = 0;
   return SW4G_OK;
}

extern "C" int sw4g_geographic_coord(const sw4g_geo* geo, double x, double y, double* lon, double* lat)
{
   if (!geo || !lon || !lat || !(geo->meters_per_degree > 0)) return SW4G_BAD_ARGUMENT;
   if (geo->const_meters_per_longitude && !(geo->meters_per_longitude > 0)) return SW4G_BAD_ARGUMENT;
   const double deg = kPi / 180.0;
   const double az = geo->az * deg;
   // latitude along the grid's rotated x axis, longitude along its y axis
   const double la = geo->lat_origin + (x * std::cos(az) - y * std::sin(az)) / geo->meters_per_degree;
   const double along = x * std::sin(az) + y * std::cos(az);
   const double lo = geo->const_meters_per_longitude
                         ? geo->lon_origin + along / geo->meters_per_longitude
                         : geo->lon_origin + along / (geo->meters_per_degree * std::cos(la * deg));
   *lat = la;
   *lon = lo;
   return SW4G_OK;
}

extern "C" int sw4g_write_usgs(const char* path, const sw4g_geo* geo, const sw4g_usgs_station* st,
                               const double* rec, long long rows, long long row_stride)
{
   if (!path || !geo || !st || rows < 0 || (rows > 0 && !rec)) return SW4G_BAD_ARGUMENT;
   const int nv = mode_values(st->mode);
   if (nv == 0 || (rows > 1 && row_stride < nv)) return SW4G_BAD_ARGUMENT;
   double lon = 0, lat = 0, gp_lon = 0, gp_lat = 0;
   if (sw4g_geographic_coord(geo, st->x, st->y, &lon, &lat) != SW4G_OK ||
       sw4g_geographic_coord(geo, st->gp_x, st->gp_y, &gp_lon, &gp_lat) != SW4G_OK)
      return SW4G_BAD_ARGUMENT;
   FILE* f = std::fopen(path, "w");
   if (!f) return SW4G_IO_ERROR;

   const int* u = st->utc;
   std::fprintf(f, "# Author: SW4\n");
   std::fprintf(f, "# Scenario: %s\n", "test");
   std::fprintf(f, "# Date: UTC  %02i/%02i/%i:%i:%i:%02i.%.3i\n", u[1], u[2], u[0], u[3], u[4], u[5], u[6]);
   std::fprintf(f, "# Bandwith (Hz): %e\n", 1.234);
   std::fprintf(f, "# Station: %s\n", st->station ? st->station : "");
   std::fprintf(f, "# Target location (WGS84 longitude, latitude) (deg): %e %e\n", lon, lat);
   std::fprintf(f, "# Actual location (WGS84 longitude, latitude) (deg): %e %e\n", gp_lon, gp_lat);
   const double dx = st->x - st->gp_x, dy = st->y - st->gp_y;
   std::fprintf(f, "# Distance from target to actual location (m): %e\n", std::sqrt(dx * dx + dy * dy));
   std::fprintf(f, "# nColumns: %i\n", nv + 1);
   std::fprintf(f, "# Column 1: Time (s)\n");
   write_column_labels(f, st->mode, st->xyz);

   int status = SW4G_OK;
   if (st->xyz || st->mode == SW4G_REC_DIV) {
      for (long long r = 0; r < rows; r++) {
         const double* v = rec + r * row_stride;
         std::fprintf(f, "%e", st->t_shift + r * st->dt);
         for (int c = 0; c < nv; c++) std::fprintf(f, " %24.17e", v[c]);
         std::fprintf(f, "\n");
      }
   } else if (st->mode == SW4G_REC_DISPLACEMENT || st->mode == SW4G_REC_VELOCITY) {
      const double deg = kPi / 180.0;
      const double ca = std::cos(kPi * geo->az / 180.0), sa = std::sin(kPi * geo->az / 180.0);
      const double cphi = std::cos(kPi * lat / 180.0), sphi = std::sin(kPi * lat / 180.0);
      const double d = (st->x * sa + st->y * ca) / cphi / geo->meters_per_degree * deg * sphi;
      double tx = sa + d * ca, ty = ca - d * sa;
      const double nrm = std::sqrt(tx * tx + ty * ty);
      tx /= nrm;
      ty /= nrm;
      for (long long r = 0; r < rows; r++) {
         const double* v = rec + r * row_stride;
         const double ns = ty * v[0] - tx * v[1];
         const double ew = sa * v[0] + ca * v[1];
         std::fprintf(f, "%e", st->t_shift + r * st->dt);
         std::fprintf(f, " %24.17e", ew);
         std::fprintf(f, " %24.17e", ns);
         std::fprintf(f, " %24.17e", -v[2]);
         std::fprintf(f, "\n");
      }
   } else {
      status = SW4G_NOT_SUPPORTED;  // curl, strains, gradient: header only
   }
   if (std::fclose(f) != 0 && status == SW4G_OK) status = SW4G_IO_ERROR;
   return status;
}
