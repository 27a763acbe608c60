// io.cu -- gauge configuration files in the reference's two formats
// (io.c:35-700), host code: the ASCII format (a header line
// "nx ny nz nt beta mass nflavs traj", then per link direction 2*mu+parity
// and half-lattice index every 3x3 matrix, rows of "(re, im)" pairs printed
// with %.18lf) and ILDG binary (LIME records with 144-byte big-endian
// headers, 8-byte padding, the "ildg-format" XML, "MD_traj", "input-file",
// "ildg-binary-data" with the links as big-endian doubles site by site,
// t slowest and x fastest, directions x, y, z, t, and an empty
// "ildg-data-lfn").  The arrays are host su3_soa[8] of the lattice given to
// ostaple_init (these functions need no GPU).
#include <cinttypes>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include "runtime.cuh"
#include "../../include/ostaple_gb300.h"

extern "C" {
// The reference's settings-file text, written into the "input-file" record
// (setting_file_parser.h:11), and the values of the ASCII header line that
// the reference takes from its fermion settings.  Weak: a host program that
// links the reference's own definitions keeps them.
__attribute__((weak)) char input_file_str[300 * 500] = "";
__attribute__((weak)) double ostaple_io_ferm_mass = 0.0;
__attribute__((weak)) int ostaple_io_nflavs = 0;
}

namespace {

typedef std::complex<double> Cd;

struct Lat {
  int n[4];
  long sizeh;
};

bool lattice(Lat* l, const char* who) {
  const ost::Geom& g = ost::host_geom();
  if (g.sizeh <= 0) {
    ost::set_error(-2, "%s: no lattice (call ostaple_init first)", who);
    return false;
  }
  l->n[0] = g.n0; l->n[1] = g.n1; l->n[2] = g.n2; l->n[3] = g.n3;
  l->sizeh = g.sizeh;
  return true;
}

long snum(const Lat& l, int x, int y, int z, int t) {
  return (x + long(l.n[0]) * (y + long(l.n[1]) * (z + long(l.n[2]) * t))) / 2;
}

// 3x3 matrix of link (dir, i), third row rebuilt as conj(r0 x r1) (rebuild3row)
struct M { Cd m[3][3]; };
M load(const Cd* u, long sh, int dir, long i) {
  M a;
  for (int r = 0; r < 2; ++r)
    for (int c = 0; c < 3; ++c) a.m[r][c] = u[(long(dir) * 9 + r * 3 + c) * sh + i];
  a.m[2][0] = std::conj(a.m[0][1] * a.m[1][2] - a.m[0][2] * a.m[1][1]);
  a.m[2][1] = std::conj(a.m[0][2] * a.m[1][0] - a.m[0][0] * a.m[1][2]);
  a.m[2][2] = std::conj(a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0]);
  return a;
}
void store(Cd* u, long sh, int dir, long i, const M& a) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) u[(long(dir) * 9 + r * 3 + c) * sh + i] = a.m[r][c];
}

bool host_little_endian() {
  const uint16_t one = 1;
  unsigned char b;
  memcpy(&b, &one, 1);
  return b == 1;
}
template <typename T> T be(T v) {   // host <-> big endian
  if (!host_little_endian()) return v;
  unsigned char b[sizeof(T)];
  memcpy(b, &v, sizeof(T));
  for (size_t k = 0; k < sizeof(T) / 2; ++k) std::swap(b[k], b[sizeof(T) - 1 - k]);
  memcpy(&v, b, sizeof(T));
  return v;
}

// LIME record header (144 bytes): magic 0x456789ab, version 1, MB/ME flags,
// payload length, 128-byte type string; all integers big endian
struct LimeHeader {
  uint32_t magic;
  uint16_t version;
  uint16_t mbme;
  uint64_t length;
  char type[128];
};
static_assert(sizeof(LimeHeader) == 144, "LIME header is 144 bytes");

bool write_record(FILE* f, const char* type, const void* data, uint64_t len) {
  LimeHeader h;
  memset(&h, 0, sizeof(h));
  const uint64_t pad = len % 8 ? 8 - len % 8 : 0;
  h.magic = be<uint32_t>(0x456789abu);
  h.version = be<uint16_t>(1);
  h.mbme = 0;
  h.length = be<uint64_t>(len + pad);   // the reference stores the padded length
  strncpy(h.type, type, sizeof(h.type) - 1);
  if (fwrite(&h, sizeof(h), 1, f) != 1) return false;
  if (len && data && fwrite(data, 1, len, f) != len) return false;
  static const char zeros[8] = {0};
  return pad == 0 || fwrite(zeros, 1, pad, f) == pad;
}

}  // namespace

extern "C" {

int print_su3_soa_ASCII(global_su3_soa* const conf_rw, const char* nomefile, int conf_id_iter,
                        double_soa* back_phases) {
  Lat l;
  if (!lattice(&l, "print_su3_soa_ASCII")) return 2;
  FILE* fp = fopen(nomefile, "w");
  if (!fp) {
    printf("ERROR, %s unreadable.\n", nomefile);
    return 2;
  }
  const Cd* u = reinterpret_cast<const Cd*>(conf_rw);
  const double* ph = reinterpret_cast<const double*>(back_phases);
  fprintf(fp, "%d %d %d %d %lf %lf %d %d\n", l.n[0], l.n[1], l.n[2], l.n[3], act_params.beta,
          ostaple_io_nflavs != 0 ? ostaple_io_ferm_mass : 0.0, ostaple_io_nflavs, conf_id_iter);
  long minuses = 0;
  for (int q = 0; q < 8; ++q)
    for (long i = 0; i < l.sizeh; ++i) {
      const M a = load(u, l.sizeh, q, i);
      int s = 1;
      if (ph && std::fabs(ph[long(q) * l.sizeh + i]) > 0.001) { s = -1; ++minuses; }
      for (int r = 0; r < 3; ++r) {
        for (int c = 0; c < 3; ++c) fprintf(fp, "(%.18lf, %.18lf)  ", s * a.m[r][c].real(), s * a.m[r][c].imag());
        fprintf(fp, "\n");
      }
      fprintf(fp, "\n");
    }
  fclose(fp);
  if (ph) {
    const long expected = long(l.n[0]) * l.n[1] * l.n[2] * l.n[3] * 3 / 2;
    if (minuses != expected) {
      printf("WRONG NUMBER OF DET=-1 MATRICES.\n");
      return 1;
    }
  }
  return 0;
}

int read_su3_soa_ASCII(global_su3_soa* conf, const char* nomefile, int* conf_id_iter) {
  Lat l;
  if (!lattice(&l, "read_su3_soa_ASCII")) return 2;
  FILE* fp = fopen(nomefile, "r");
  if (!fp) {
    printf("Gauge configuration file %s not readable.\n", nomefile);
    *conf_id_iter = -1;
    return 1;
  }
  int n[4], nfl;
  double beta, mass;
  if (fscanf(fp, "%d %d %d %d %lf %lf %d %d\n", &n[0], &n[1], &n[2], &n[3], &beta, &mass, &nfl, conf_id_iter) != 8) {
    fclose(fp);
    return 2;
  }
  if (n[0] != l.n[0] || n[1] != l.n[1] || n[2] != l.n[2] || n[3] != l.n[3]) {
    printf("Error, configuration dimensions not compatible with code.\n");
    fclose(fp);
    return 2;
  }
  Cd* u = reinterpret_cast<Cd*>(conf);
  for (int q = 0; q < 8; ++q)
    for (long i = 0; i < l.sizeh; ++i) {
      M a;
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          double re, im;
          const char* fmt = c < 2 ? "(%lf, %lf) " : "(%lf, %lf)\n";
          if (fscanf(fp, fmt, &re, &im) != 2) {
            fclose(fp);
            return 2;
          }
          a.m[r][c] = Cd(re, im);
        }
      // a matrix written with a staggered sign has determinant -1: undo it
      // (io.c:160-175)
      const Cd det = a.m[0][0] * (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1]) -
                     a.m[0][1] * (a.m[1][0] * a.m[2][2] - a.m[1][2] * a.m[2][0]) +
                     a.m[0][2] * (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]);
      if (std::fabs(1.0 + det.real()) < 0.005)
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) a.m[r][c] = -a.m[r][c];
      store(u, l.sizeh, q, i, a);
    }
  fclose(fp);
  return 0;
}

int print_su3_soa_ildg_binary(global_su3_soa* conf, const char* nomefile, int conf_id_iter) {
  Lat l;
  if (!lattice(&l, "print_su3_soa_ildg_binary")) return 2;
  FILE* fp = fopen(nomefile, "w");
  if (!fp) {
    printf("ERROR, %s unreadable.\n", nomefile);
    return 2;
  }
  char fmt[1000];
  snprintf(fmt, sizeof(fmt),
           "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n"
           "            <ildgFormat xmlns=\"http://www.lqcd.org/ildg\"\n"
           "            xmlns:xsi=\"http://www.w3.org/2001/XMLSchema-instance\"\n"
           "            xsi:schemaLocation=\"http://www.lqcd.org/ildg filefmt.xsd\">\n"
           "            <version>1.0</version>\n"
           "            <field>su3gauge</field>\n"
           "            <precision>64</precision>\n"
           "            <lx>%d</lx>\n"
           "            <ly>%d</ly>\n"
           "            <lz>%d</lz>\n"
           "            <lt>%d</lt>\n"
           "            </ildgFormat>",
           l.n[0], l.n[1], l.n[2], l.n[3]);
  char traj[32];
  snprintf(traj, sizeof(traj), "%d", conf_id_iter);
  bool ok = write_record(fp, "ildg-format", fmt, strlen(fmt)) && write_record(fp, "MD_traj", traj, strlen(traj)) &&
            write_record(fp, "input-file", input_file_str, strlen(input_file_str));
  // ildg-binary-data: per site (t, z, y, x; x fastest), directions x, y, z, t,
  // 3x3 complex big-endian doubles, row by row
  const uint64_t len = uint64_t(l.n[0]) * l.n[1] * l.n[2] * l.n[3] * 4 * 3 * 3 * 2 * 8;
  std::vector<double> buf(size_t(l.n[0]) * 4 * 18);
  const Cd* u = reinterpret_cast<const Cd*>(conf);
  if (ok) {
    LimeHeader h;
    memset(&h, 0, sizeof(h));
    h.magic = be<uint32_t>(0x456789abu);
    h.version = be<uint16_t>(1);
    h.length = be<uint64_t>(len);
    strncpy(h.type, "ildg-binary-data", sizeof(h.type) - 1);
    ok = fwrite(&h, sizeof(h), 1, fp) == 1;
  }
  for (int t = 0; t < l.n[3] && ok; ++t)
    for (int z = 0; z < l.n[2] && ok; ++z)
      for (int y = 0; y < l.n[1] && ok; ++y) {
        size_t k = 0;
        for (int x = 0; x < l.n[0]; ++x) {
          const int p = (x + y + z + t) & 1;
          const long i = snum(l, x, y, z, t);
          for (int mu = 0; mu < 4; ++mu) {
            const M a = load(u, l.sizeh, 2 * mu + p, i);
            for (int r = 0; r < 3; ++r)
              for (int c = 0; c < 3; ++c) {
                buf[k++] = be<double>(a.m[r][c].real());
                buf[k++] = be<double>(a.m[r][c].imag());
              }
          }
        }
        ok = fwrite(buf.data(), sizeof(double), k, fp) == k;
      }
  ok = ok && write_record(fp, "ildg-data-lfn", nullptr, 0);
  fclose(fp);
  if (!ok) {
    printf("Error in writing file: %s\n", nomefile);
    return 2;
  }
  return 0;
}

int read_su3_soa_ildg_binary(global_su3_soa* conf, const char* nomefile, int* conf_id_iter) {
  Lat l;
  if (!lattice(&l, "read_su3_soa_ildg_binary")) return 2;
  *conf_id_iter = 1000;
  FILE* fg = fopen(nomefile, "r");
  if (!fg) {
    printf("Gauge configuration ILDG file %s not readable.\n", nomefile);
    *conf_id_iter = -1;
    return 1;
  }
  // walk the records (io.c:252-300)
  long fmt_at = -1, bin_at = -1, traj_at = -1;
  uint64_t fmt_len = 0, traj_len = 0;
  for (int k = 0; k < 64 && (fmt_at < 0 || bin_at < 0); ++k) {
    LimeHeader h;
    if (fread(&h, sizeof(h), 1, fg) != 1) break;
    h.type[127] = 0;
    const uint64_t len = be<uint64_t>(h.length);
    const long at = ftell(fg);
    if (!strcmp(h.type, "ildg-format")) { fmt_at = at; fmt_len = len; }
    if (!strcmp(h.type, "ildg-binary-data")) bin_at = at;
    if (!strcmp(h.type, "MD_traj")) { traj_at = at; traj_len = len; }
    const uint64_t skip = len + (len % 8 ? 8 - len % 8 : 0);
    if (fseek(fg, long(skip), SEEK_CUR) != 0) break;
  }
  if (fmt_at < 0 || bin_at < 0) {
    printf("Error in reading file: ildg-format or ildg-binary-data record missing\n");
    fclose(fg);
    return 2;
  }
  std::string fmt(size_t(fmt_len), '\0');
  fseek(fg, fmt_at, SEEK_SET);
  if (fread(&fmt[0], 1, fmt.size(), fg) != fmt.size()) { fclose(fg); return 2; }
  const char* tags[4] = {"<lx>", "<ly>", "<lz>", "<lt>"};
  for (int d = 0; d < 4; ++d) {
    const size_t at = fmt.find(tags[d]);
    if (at == std::string::npos) {
      printf("Error, lx,ly,lz or lt not found in \"ildg-format\"\n");
      fclose(fg);
      return 2;
    }
    if (atoi(fmt.c_str() + at + 4) != l.n[d]) {
      printf("Error, Configuration dimensions not compatible with input file.\n");
      fclose(fg);
      return 2;
    }
  }
  if (traj_at >= 0 && traj_len > 0) {
    fseek(fg, traj_at, SEEK_SET);
    if (fscanf(fg, "%d", conf_id_iter) != 1) { fclose(fg); return 2; }
  } else {
    *conf_id_iter = 1;
  }
  fseek(fg, bin_at, SEEK_SET);
  Cd* u = reinterpret_cast<Cd*>(conf);
  std::vector<double> buf(size_t(l.n[0]) * 4 * 18);
  for (int t = 0; t < l.n[3]; ++t)
    for (int z = 0; z < l.n[2]; ++z)
      for (int y = 0; y < l.n[1]; ++y) {
        if (fread(buf.data(), sizeof(double), buf.size(), fg) != buf.size()) {
          printf("Error in reading file: %s\n", nomefile);
          fclose(fg);
          return 2;
        }
        size_t k = 0;
        for (int x = 0; x < l.n[0]; ++x) {
          const int p = (x + y + z + t) & 1;
          const long i = snum(l, x, y, z, t);
          for (int mu = 0; mu < 4; ++mu) {
            M a;
            for (int r = 0; r < 3; ++r)
              for (int c = 0; c < 3; ++c) {
                const double re = be<double>(buf[k++]);
                const double im = be<double>(buf[k++]);
                a.m[r][c] = Cd(re, im);
              }
            // the reference keeps rows 0-1 and rebuilds row 2 (rebuild3row)
            a.m[2][0] = std::conj(a.m[0][1] * a.m[1][2] - a.m[0][2] * a.m[1][1]);
            a.m[2][1] = std::conj(a.m[0][2] * a.m[1][0] - a.m[0][0] * a.m[1][2]);
            a.m[2][2] = std::conj(a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0]);
            store(u, l.sizeh, 2 * mu + p, i, a);
          }
        }
      }
  fclose(fg);
  return 0;
}

}  // extern "C"
