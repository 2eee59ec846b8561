// Receiver files in the USGS text format and as binary SAC traces, and the grid's
// geographic mapping (host code, no device work).
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
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

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

// grid components to (east-west, north-south) at a requested location (x, y) of
// latitude lat: ew = sa u0 + ca u1, ns = ty u0 - tx u1
struct Rotation {
   double sa, ca, tx, ty;
};
Rotation rotation(const sw4g_geo& geo, double x, double y, double lat)
{
   Rotation r;
   const double deg = kPi / 180.0;
   r.ca = std::cos(kPi * geo.az / 180.0);
   r.sa = std::sin(kPi * geo.az / 180.0);
   const double cphi = std::cos(kPi * lat / 180.0), sphi = std::sin(kPi * lat / 180.0);
   const double d = (x * r.sa + y * r.ca) / cphi / geo.meters_per_degree * deg * sphi;
   r.tx = r.sa + d * r.ca;
   r.ty = r.ca - d * r.sa;
   const double nrm = std::sqrt(r.tx * r.tx + r.ty * r.ty);
   r.tx /= nrm;
   r.ty /= nrm;
   return r;
}

// ---------------------------------------------------------------------------
// Binary SAC (version 6 header): 70 FP32 words, 40 integer words (the last five
// logicals), 24 eight-character fields (KEVNM spans two), 632 bytes, then the
// samples as FP32.  Unset words hold -12345 ("-12345  " for text).
constexpr int kSacF = 70, kSacI = 40, kSacK = 24;
enum SacF { F_DELTA = 0, F_DEPMIN = 1, F_DEPMAX = 2, F_B = 5, F_E = 6, F_O = 7, F_STLA = 31, F_STLO = 32,
            F_EVLA = 35, F_EVLO = 36, F_EVDP = 38, F_DEPMEN = 56, F_CMPAZ = 57, F_CMPINC = 58 };
enum SacI { I_NZYEAR = 0, I_NZJDAY = 1, I_NZHOUR = 2, I_NZMIN = 3, I_NZSEC = 4, I_NZMSEC = 5, I_NVHDR = 6,
            I_NORID = 7, I_NEVID = 8, I_NPTS = 9, I_IFTYPE = 15, I_LEVEN = 35, I_LOVROK = 37, I_LCALDA = 38 };
enum SacK { K_KSTNM = 0, K_KCMPNM = 20 };

struct SacHeader {
   float f[kSacF];
   int32_t i[kSacI];
   char k[kSacK][8];
};
static_assert(sizeof(SacHeader) == 632, "SAC header is 632 bytes");

// a fresh header: everything unset but the version (6), the origin and event ids
// (0), the logicals (false), then an evenly sampled time series (IFTYPE = ITIME = 1,
// LEVEN, LOVROK, LCALDA true)
void sac_new(SacHeader& h)
{
   for (float& x : h.f) x = -12345.0f;
   for (int32_t& x : h.i) x = -12345;
   for (auto& x : h.k) std::memcpy(x, "-12345  ", 8);
   h.i[I_NVHDR] = 6;
   h.i[I_NORID] = h.i[I_NEVID] = 0;
   for (int q = 35; q < 40; q++) h.i[q] = 0;
   h.i[I_IFTYPE] = 1;
   h.i[I_LEVEN] = h.i[I_LOVROK] = h.i[I_LCALDA] = 1;
}

// first 8 characters, blank padded
void sac_text(char out[8], const char* s)
{
   const size_t n = s ? std::strlen(s) : 0;
   for (size_t c = 0; c < 8; c++) out[c] = c < n ? s[c] : ' ';
}

int days_in_month(int year, int month)
{
   if (month == 2) return 28 + ((year % 400 == 0) || (year % 4 == 0 && year % 100 != 0));
   return (month == 4 || month == 6 || month == 9 || month == 11) ? 30 : 31;
}

// one component's file
int sac_write_one(const std::string& path, const float* y, int npts, float btime, float dt, const char* name,
                  float cmpinc, float cmpaz, const sw4g_usgs_station& st, const sw4g_sac_event& ev,
                  double rec_lat, double rec_lon)
{
   SacHeader h;
   sac_new(h);
   float ymax = -1.0e+38f, ymin = 1.0e+38f;
   double sum = 0;
   for (int r = 0; r < npts; r++) {
      if (y[r] > ymax) ymax = y[r];
      if (y[r] < ymin) ymin = y[r];
      sum += y[r];
   }
   h.f[F_DEPMAX] = ymax;
   h.f[F_DEPMIN] = ymin;
   h.f[F_DEPMEN] = npts > 0 ? (float)(sum / npts) : -12345.0f;
   h.i[I_NPTS] = npts;
   h.f[F_DELTA] = dt;
   h.f[F_B] = btime;
   const float steps = (float)(npts - 1);
   const float span = steps * dt;
   h.f[F_E] = btime + span;
   const int* u = st.utc;
   int jday = u[2];
   for (int m = 1; m < u[1]; m++) jday += days_in_month(u[0], m);
   h.i[I_NZYEAR] = u[0];
   h.i[I_NZJDAY] = jday;
   h.i[I_NZHOUR] = u[3];
   h.i[I_NZMIN] = u[4];
   h.i[I_NZSEC] = u[5];
   h.i[I_NZMSEC] = u[6];
   sac_text(h.k[K_KCMPNM], name);
   h.f[F_STLA] = (float)rec_lat;
   h.f[F_STLO] = (float)rec_lon;
   h.f[F_EVLA] = (float)ev.lat;
   h.f[F_EVLO] = (float)ev.lon;
   h.f[F_EVDP] = (float)(ev.depth / 1000.0);
   h.f[F_O] = (float)ev.time_offset;
   h.f[F_CMPINC] = cmpinc;
   h.f[F_CMPAZ] = cmpaz;
   sac_text(h.k[K_KSTNM], st.station);
   FILE* f = std::fopen(path.c_str(), "wb");
   if (!f) return SW4G_IO_ERROR;
   bool ok = std::fwrite(&h, sizeof h, 1, f) == 1;
   if (npts > 0) ok = ok && std::fwrite(y, sizeof(float), (size_t)npts, f) == (size_t)npts;
   ok = std::fclose(f) == 0 && ok;
   return ok ? SW4G_OK : SW4G_IO_ERROR;
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
      const Rotation q = rotation(*geo, st->x, st->y, lat);
      const double sa = q.sa, ca = q.ca, tx = q.tx, ty = q.ty;
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

extern "C" int sw4g_write_sac(const char* prefix, const sw4g_geo* geo, const sw4g_usgs_station* st,
                              const sw4g_sac_event* ev, const double* rec, long long rows, long long row_stride,
                              int flush_subnormals)
{
   if (!prefix || !geo || !st || !ev || rows < 0 || rows > 0x7fffffffLL || (rows > 0 && !rec))
      return SW4G_BAD_ARGUMENT;
   const int nv = mode_values(st->mode);
   if (nv == 0 || (rows > 1 && row_stride < nv)) return SW4G_BAD_ARGUMENT;
   double lon = 0, lat = 0;
   if (sw4g_geographic_coord(geo, st->x, st->y, &lon, &lat) != SW4G_OK) return SW4G_BAD_ARGUMENT;
   // per value: file suffix, component name, inclination, azimuth (the grid's x
   // axis at az, y at az + 90, up-down 180 from vertical; geographic components
   // east 90, north 0, up 0)
   struct Comp {
      const char *suffix, *name;
      int kind;  // 0: (90, az), 1: (90, az + 90), 2: (updown, 0)
   };
   static const Comp disp[3] = {{"x", "X", 0}, {"y", "Y", 1}, {"z", "Z", 2}};
   static const Comp disp_g[3] = {{"e", "EW", 0}, {"n", "NS", 1}, {"u", "UP", 2}};
   static const Comp velo[3] = {{"xv", "Vx", 0}, {"yv", "Vy", 1}, {"zv", "Vz", 2}};
   static const Comp velo_g[3] = {{"ev", "Vew", 0}, {"nv", "Vns", 1}, {"uv", "Vup", 2}};
   static const Comp div[1] = {{"div", "Div", 0}};
   static const Comp curl[3] = {{"curlx", "Curlx", 0}, {"curly", "Curly", 1}, {"curlz", "Curlz", 2}};
   static const Comp strain[6] = {{"xx", "Uxx", 0}, {"yy", "Uyy", 1}, {"zz", "Uzz", 2},
                                  {"xy", "Uxy", 0}, {"xz", "Uxz", 0}, {"yz", "Uyz", 0}};
   static const Comp grad[9] = {{"duxdx", "DUXDX", 0}, {"duxdy", "DUXDY", 0}, {"duxdz", "DUXDZ", 0},
                                {"duydx", "DUYDX", 0}, {"duydy", "DUYDY", 1}, {"duydz", "DUYDZ", 0},
                                {"duzdx", "DUZDX", 0}, {"duzdy", "DUZDY", 0}, {"duzdz", "DUZDZ", 2}};
   const bool geo_comp = !st->xyz && (st->mode == SW4G_REC_DISPLACEMENT || st->mode == SW4G_REC_VELOCITY ||
                                      st->mode == SW4G_REC_CURL);
   const Comp* comps = nullptr;
   switch (st->mode) {
   case SW4G_REC_DISPLACEMENT: comps = st->xyz ? disp : disp_g; break;
   case SW4G_REC_VELOCITY: comps = st->xyz ? velo : velo_g; break;
   case SW4G_REC_DIV: comps = div; break;
   case SW4G_REC_CURL: comps = curl; break;
   case SW4G_REC_STRAINS: comps = strain; break;
   default: comps = grad; break;
   }
   // displacement and velocity in geographic components are east, north and up;
   // everything else keeps the grid's axes
   const bool geo_axes = !st->xyz && (st->mode == SW4G_REC_DISPLACEMENT || st->mode == SW4G_REC_VELOCITY);
   const float az_x = geo_axes ? 90.0f : (float)geo->az;
   const float az_y = geo_axes ? 0.0f : (float)(geo->az + 90.0);
   const float updown = geo_axes ? 0.0f : 180.0f;
   const int n = (int)rows;
   std::vector<float> y((size_t)nv * (size_t)n);
   for (int r = 0; r < n; r++)
      for (int c = 0; c < nv; c++) y[(size_t)c * n + r] = (float)rec[(long long)r * row_stride + c];
   // an FP32 result below the smallest normal becomes a zero of its sign
   auto flush = [&](float v) { return std::fabs(v) < FLT_MIN ? std::copysign(0.0f, v) : v; };
   if (flush_subnormals)
      for (float& v : y) v = flush(v);
   if (geo_comp) {  // rotated from the FP32 values, in FP64, rounded to FP32
      const Rotation q = rotation(*geo, st->x, st->y, lat);
      for (int r = 0; r < n; r++) {
         const float u0 = y[r], u1 = y[(size_t)n + r], u2 = y[2 * (size_t)n + r];
         float ns = (float)(q.ty * u0 - q.tx * u1), ew = (float)(q.sa * u0 + q.ca * u1);
         if (flush_subnormals) {
            ns = flush(ns);
            ew = flush(ew);
         }
         y[(size_t)n + r] = ns;
         y[r] = ew;
         y[2 * (size_t)n + r] = -u2;
      }
   }
   const float btime = (float)st->t_shift, dt = (float)st->dt;
   for (int c = 0; c < nv; c++) {
      const Comp& k = comps[c];
      const float inc = k.kind == 2 ? updown : 90.0f;
      const float az = k.kind == 0 ? az_x : k.kind == 1 ? az_y : 0.0f;
      const int s = sac_write_one(std::string(prefix) + k.suffix, y.data() + (size_t)c * n, n, btime, dt, k.name,
                                  inc, az, *st, *ev, lat, lon);
      if (s != SW4G_OK) return s;
   }
   return SW4G_OK;
}
