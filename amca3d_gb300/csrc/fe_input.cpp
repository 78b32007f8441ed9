// fe_input.cpp — see fe_input.h.
#include "fe_input.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <fstream>
#include <sstream>
#include <stdexcept>

namespace amca {

namespace {

// std::getline over a file's bytes with the stream's eof flag: eof is raised
// when a read reaches the end of the data (no newline, or nothing left). The
// file is read in chunks, so a frame file of any size streams.
class LineReader {
 public:
  explicit LineReader(const std::string &path) : f_(path.c_str(), std::ios::in | std::ios::binary) {
    if (!f_) throw std::runtime_error("fail to open the specified file " + path);
  }
  bool eof() const { return eof_; }
  void getline(std::string &line) {
    line.clear();
    for (;;) {
      if (pos_ >= buf_.size() && !refill()) {
        if (line.empty() && !partial_) eof_ = true;  // nothing left at all
        else eof_ = true;                             // the last line had no newline
        partial_ = false;
        return;
      }
      const size_t nl = buf_.find('\n', pos_);
      if (nl == std::string::npos) {
        line.append(buf_, pos_, std::string::npos);
        pos_ = buf_.size();
        partial_ = true;
        continue;
      }
      line.append(buf_, pos_, nl - pos_);
      pos_ = nl + 1;
      partial_ = false;
      if (pos_ >= buf_.size()) refill_at_end();
      return;
    }
  }

 private:
  bool refill() {
    buf_.resize(kChunk);
    f_.read(&buf_[0], (std::streamsize)kChunk);
    buf_.resize((size_t)f_.gcount());
    pos_ = 0;
    return !buf_.empty();
  }
  // after a line that ended exactly at the end of the buffer: fetch the next
  // chunk now, so that "nothing left" is known at the next call
  void refill_at_end() {
    if (!refill()) buf_.clear();
  }
  static constexpr size_t kChunk = size_t(16) << 20;
  std::ifstream f_;
  std::string buf_;
  size_t pos_ = 0;
  bool eof_ = false, partial_ = false;
};

}  // namespace

struct FrameReader::Impl {
  LineReader L;
  FeConfig fe;
  double toff = 0.0;
  std::vector<double> cur;
  explicit Impl(const std::string &path, const FeConfig &c) : L(path), fe(c) {}
};

FrameReader::~FrameReader() = default;

// load_mesh_and_first_two_steps_results_from_txt_file: title, the first
// subtitle (node ranges, time) and the first frame with the coordinates.
FrameReader::FrameReader(const std::string &path, const FeConfig &fe) : impl_(new Impl(path, fe)) {
  LineReader &L = impl_->L;
  std::string line;
  int dummy[2] = {0, 0};
  double time[2] = {0, 0};
  int range[6] = {0, 0, 0, 0, 0, 0};
  const int skip = fe.title_lines + fe.subtitle_lines;
  for (int count = 0; count < skip; ++count) {
    L.getline(line);
    if (count == fe.title_lines + 3) {
      std::istringstream iss(line);
      iss >> dummy[0] >> dummy[1] >> time[0] >> time[1];
      for (int i = 0; i < 6; i++) iss >> range[i];
    }
  }
  impl_->toff = time[0];
  FeFrames &fr = head_;
  for (int i = 0; i < 3; i++) fr.nn[i] = range[2 * i + 1] - range[2 * i] + 1;
  fr.nnodes = (int64_t)fr.nn[0] * fr.nn[1] * fr.nn[2];
  if (fr.nnodes == 1 || fr.nn[0] < 2 || fr.nn[1] < 2 || fr.nn[2] < 2)
    throw std::runtime_error("fail to read temperature file, please check the file type and the lines of title!!");
  fr.coord.resize(3 * (size_t)fr.nnodes);
  std::vector<double> &cur = impl_->cur;
  cur.assign((size_t)fr.nnodes, 0.0);
  for (int64_t n = 0; n < fr.nnodes; ++n) {
    L.getline(line);
    std::istringstream iss(line);
    for (int d = 0; d < 3; d++) {
      double x = 0;
      iss >> x;
      x += fe.offset[d];
      x *= fe.length_scale;
      fr.coord[3 * n + d] = x;
    }
    double t = 0;
    iss >> t;
    cur[n] = t;
  }
  fr.times.push_back(0.0);
  fr.theta = cur;
  fr.nframes = 1;
  read_ = 1;
}

// load_next_step_nodal_data: one more frame, or false at the end of the file
// or at a malformed frame (bad() tells which).
bool FrameReader::next(double *out, double &t) {
  if (done_) return false;
  LineReader &L = impl_->L;
  const FeConfig &fe = impl_->fe;
  std::vector<double> &cur = impl_->cur;  // keeps the previous frame's values where a line lacks one
  const int64_t nnodes = head_.nnodes;
  std::string line;
  int64_t count = 0;
  double tnew = 0;
  double result = 0;  // keeps the previous line's value when a line lacks it
  while (count < fe.subtitle_lines + nnodes) {
    if (L.eof()) {
      done_ = true;
      return false;
    }
    L.getline(line);
    if (count == 0 && line != "\r" && line != "") {
      bad_ = true;
      bad_msg_ = "fail to read next step temperature file, please check title of line!!";
      done_ = true;
      return false;
    }
    if (count == 3) {
      std::istringstream iss(line);
      int d0 = 0, d1 = 0;
      double t0 = 0, t1 = 0;
      iss >> d0 >> d1 >> t0 >> t1;
      tnew = t0;
    }
    if (count >= fe.subtitle_lines) {
      std::istringstream iss(line);
      double c0, c1, c2;
      iss >> c0 >> c1 >> c2 >> result;
      cur[count - fe.subtitle_lines] = result;
    }
    count++;
  }
  t = (tnew - impl_->toff) * fe.time_scale;
  memcpy(out, cur.data(), (size_t)nnodes * sizeof(double));
  ++read_;
  return true;
}

FeFrames read_fe_frames(const std::string &path, const FeConfig &fe) {
  FrameReader rd(path, fe);
  FeFrames fr = rd.head();
  std::vector<double> cur((size_t)fr.nnodes);
  double t = 0;
  while (rd.next(cur.data(), t)) {
    fr.times.push_back(t);
    fr.theta.insert(fr.theta.end(), cur.begin(), cur.end());
    fr.nframes++;
  }
  if (rd.bad()) {
    fr.bad_frame = fr.nframes;
    fr.bad_msg = rd.bad_msg();
  }
  if (fr.nframes < 2) {
    if (fr.bad_frame == 1) throw std::runtime_error(fr.bad_msg);
    throw std::runtime_error("the temperature file holds fewer than two frames");
  }
  return fr;
}

FeFrames fe_frames_from_arrays(const int32_t nodes[3], const double *coords, int64_t nframes, const double *times,
                               const double *theta, const FeConfig &fe) {
  FeFrames fr;
  for (int i = 0; i < 3; ++i) fr.nn[i] = nodes[i];
  if (fr.nn[0] < 2 || fr.nn[1] < 2 || fr.nn[2] < 2) throw std::invalid_argument("at least 2 nodes per axis");
  if (nframes < 2) throw std::invalid_argument("at least two frames");
  fr.nnodes = (int64_t)fr.nn[0] * fr.nn[1] * fr.nn[2];
  fr.coord.resize(3 * (size_t)fr.nnodes);
  for (int64_t n = 0; n < fr.nnodes; ++n)
    for (int d = 0; d < 3; ++d) {
      double x = coords[3 * n + d];
      x += fe.offset[d];
      x *= fe.length_scale;
      fr.coord[3 * n + d] = x;
    }
  fr.times.resize((size_t)nframes);
  fr.times[0] = 0.0;
  for (int64_t f = 1; f < nframes; ++f) fr.times[f] = (times[f] - times[0]) * fe.time_scale;
  fr.theta.assign(theta, theta + (size_t)nframes * fr.nnodes);
  fr.nframes = nframes;
  return fr;
}

RestartData read_restart(const std::string &file_name) {
  const size_t dot = file_name.find_last_of('.');
  const std::string path = file_name.substr(0, dot) + "0.txt";
  std::ifstream in(path.c_str(), std::ios::in);
  if (!in) throw std::runtime_error("fail to open the specified file " + path);
  RestartData r;
  std::string line;
  std::getline(in, line);
  std::getline(in, line);
  {
    std::istringstream iss(line);
    int nc = 0, no = 0, ng = 0, ne = 0;
    double X, Y, Z, nx, ny, nz, dcell;
    iss >> nc >> no >> ng >> ne >> X >> Y >> Z >> nx >> ny >> nz >> dcell;
    r.ncells = nc;
    r.norient = no;
    r.ngrains = ng;
    r.expected = ne;
  }
  if (r.ncells < 0 || r.norient < 0 || r.ngrains < 0) throw std::runtime_error("bad restart header in " + path);
  r.grain.assign((size_t)r.ncells, -1);
  r.orient.assign((size_t)r.ncells, -1);
  r.melted.assign((size_t)r.ncells, 0);
  r.dtc.assign((size_t)r.ncells, -1.0);
  std::getline(in, line);
  for (int64_t count = 0; count < r.ncells;) {
    if (!std::getline(in, line)) throw std::runtime_error("restart file ends inside the cell list: " + path);
    if (!line.size()) continue;
    std::istringstream iss(line);
    int id = -1, g = -1, o = -1;
    bool m = false;
    double dt = -1;
    iss >> id >> g >> o >> m >> dt;
    if (id < 0 || id >= r.ncells) throw std::runtime_error("restart cell id out of range in " + path);
    r.grain[id] = g;
    r.orient[id] = o;
    r.melted[id] = m ? 1 : 0;
    r.dtc[id] = dt;
    count++;
  }
  std::getline(in, line);
  r.euler.resize(3 * (size_t)r.norient);
  for (int64_t count = 0; count < r.norient;) {
    if (!std::getline(in, line)) throw std::runtime_error("restart file ends inside the orientation list: " + path);
    if (!line.size()) continue;
    std::istringstream iss(line);
    int id = -1;
    double e[3] = {0, 0, 0};
    iss >> id >> e[0] >> e[1] >> e[2];
    if (id != count) throw std::runtime_error("restart orientation ids must be 0..n-1 in order: " + path);
    for (int a = 0; a < 3; ++a) r.euler[3 * count + a] = e[a];
    count++;
  }
  std::getline(in, line);
  r.gcell.resize((size_t)r.ngrains);
  r.gori.resize((size_t)r.ngrains);
  for (int64_t count = 0; count < r.ngrains;) {
    if (!std::getline(in, line)) throw std::runtime_error("restart file ends inside the grain list: " + path);
    if (!line.size()) continue;
    std::istringstream iss(line);
    int id = -1, cell = -1, o = -1;
    double x, y, z;
    iss >> id >> cell >> x >> y >> z >> o;
    if (o < 0 || o >= r.norient) throw std::runtime_error("restart grain orientation out of range: " + path);
    r.gcell[count] = cell;
    r.gori[count] = o;
    count++;
  }
  return r;
}

namespace {
inline double mv_min(double a, double b) { return ((a) < (b)) ? (a) : (b); }  // __min (MapVoxelManager.cpp:11)
inline double mv_max(double a, double b) { return ((a) > (b)) ? (a) : (b); }  // __max (MapVoxelManager.cpp:10)
}  // namespace

VoxelMapPlan plan_voxel_map(const FeFrames &fr, const PlainConfig &ca, const TransferConfig &tr) {
  VoxelMapPlan p;
  const int64_t ne = fr.nelem();
  p.erange.resize(6 * (size_t)ne);
  for (int64_t e = 0; e < ne; ++e) {  // get_cell_xyz_min_max (:262-289)
    int64_t nid[8];
    fe_elem_nodes(fr.nn, e, nid);
    double *r = &p.erange[6 * e];
    for (int i = 0; i < 3; i++) {
      r[2 * i] = 1.0e8;
      r[2 * i + 1] = -1.0e8;
    }
    for (int n = 0; n < 8; n++)
      for (int d = 0; d < 3; d++) {
        const double c = fr.coord[3 * nid[n] + d];
        r[2 * d] = mv_min(r[2 * d], c);
        r[2 * d + 1] = mv_max(r[2 * d + 1], c);
      }
  }
  // get_CA_domain_xyz_min_max (:198-256), single rank: start offsets 0
  const double h = ca.h;
  const int nxg = ca.nx + 2, nyg = ca.ny + 2, nzg = ca.nz + 2;
  double *mm = p.mm;
  mm[0] = (0 - 1) * h + ca.x0;
  mm[2] = (0 - 1) * h + ca.y0;
  mm[4] = (0 - 1) * h + ca.z0;
  mm[1] = mm[0] + nxg * h;
  mm[3] = mm[2] + nyg * h;
  mm[5] = mm[4] + nzg * h;
  double cur[6];
  for (int c = 0; c < 6; ++c) cur[c] = mm[c];
  for (int64_t e = 0; e < ne; ++e) {
    int64_t nid[8];
    fe_elem_nodes(fr.nn, e, nid);
    bool overlap = false;
    for (int n = 0; n < 8 && !overlap; n++) {
      const double *c = &fr.coord[3 * nid[n]];
      overlap = c[0] >= mm[0] && c[0] <= mm[1] && c[1] >= mm[2] && c[1] <= mm[3] && c[2] >= mm[4] && c[2] <= mm[5];
    }
    if (overlap) {
      const double *r = &p.erange[6 * e];
      for (int d = 0; d < 3; d++) {
        cur[2 * d] = mv_min(cur[2 * d], r[2 * d]);
        cur[2 * d + 1] = mv_max(cur[2 * d + 1], r[2 * d + 1]);
      }
    }
  }
  for (int c = 0; c < 6; ++c) mm[c] = cur[c];
  for (int i = 0; i < 3; i++) {  // execute_with_focus_on_CA_region (:150-157)
    p.dbin[i] = tr.bin[i] * h;
    p.nbin[i] = (int)ceil((mm[i * 2 + 1] - mm[i * 2]) / p.dbin[i]);
    if (p.nbin[i] < 1) p.nbin[i] = 1;
  }
  const int64_t nb = (int64_t)p.nbin[0] * p.nbin[1] * p.nbin[2];
  // attach_elements (:294-352)
  p.around.assign((size_t)fr.nnodes, 0);
  p.bin_start.assign((size_t)nb + 1, 0);
  std::vector<int64_t> fill;
  for (int pass = 0; pass < 2; ++pass) {
    if (pass == 1) {
      for (int64_t b = 0; b < nb; ++b) p.bin_start[b + 1] += p.bin_start[b];
      p.bin_elems.resize((size_t)p.bin_start[nb]);
      fill.assign(p.bin_start.begin(), p.bin_start.end() - 1);
    }
    for (int64_t e = 0; e < ne; ++e) {
      const double *r = &p.erange[6 * e];
      bool inside = true;
      for (int c = 0; c < 3; c++)
        if (r[c * 2] < mm[c * 2] || r[c * 2 + 1] > mm[c * 2 + 1]) {
          inside = false;
          break;
        }
      if (!inside) continue;
      if (pass == 0) {
        int64_t nid[8];
        fe_elem_nodes(fr.nn, e, nid);
        for (int n = 0; n < 8; n++) p.around[nid[n]] = 1;
      }
      const int imin = (int)floor((r[0] - mm[0]) / p.dbin[0]), imax = (int)ceil((r[1] - mm[0]) / p.dbin[0]);
      const int jmin = (int)floor((r[2] - mm[2]) / p.dbin[1]), jmax = (int)ceil((r[3] - mm[2]) / p.dbin[1]);
      const int kmin = (int)floor((r[4] - mm[4]) / p.dbin[2]), kmax = (int)ceil((r[5] - mm[4]) / p.dbin[2]);
      for (int kk = kmin; kk < kmax; kk++)
        for (int jj = jmin; jj < jmax; jj++)
          for (int ii = imin; ii < imax; ii++) {
            const int64_t ind = ii + (int64_t)jj * p.nbin[0] + (int64_t)kk * p.nbin[0] * p.nbin[1];
            if (ind < 0 || ind >= nb) continue;  // inside elements stay within the bins
            if (pass == 0)
              p.bin_start[ind + 1]++;
            else
              p.bin_elems[fill[ind]++] = (int32_t)e;
          }
    }
  }
  return p;
}

}  // namespace amca
