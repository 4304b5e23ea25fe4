// Core host utilities: error text, settings parsing, device buffers, counter-based
// hashing, GLL basis (Newton iteration on Legendre polynomials), and the Hessenberg
// eigenvalue solve used by the Arnoldi spectral-radius estimates.
#include "objects.hpp"

#include <algorithm>
#include <atomic>
#include <cctype>
#include <cmath>
#include <sstream>

namespace lpg {

static thread_local std::string g_last_error;

int set_error(int status, const std::string& msg) {
  g_last_error = msg;
  return status;
}

}  // namespace lpg

extern "C" const char* lpg_last_error(void) { return lpg::g_last_error.c_str(); }

namespace lpg {

// ---------------------------------------------------------------- settings
static std::string trim(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) a++;
  while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
  return s.substr(a, b - a);
}

// Keys of this path (ellipticSettings.cpp:57-98, meshSettings.cpp:35-90,
// parAlmondSettings.cpp:33-60, platformSettings.cpp:30-53) plus this library's additions.
static const char* kKnownKeys[] = {
    "FORMAT", "DATA FILE", "MESH FILE", "MESH DIMENSION", "ELEMENT TYPE", "ELEMENT MAP",
    "BOX NX", "BOX NY", "BOX NZ", "BOX GLOBAL NX", "BOX GLOBAL NY", "BOX GLOBAL NZ", "BOX DIMX",
    "BOX DIMY", "BOX DIMZ", "BOX BOUNDARY FLAG", "POLYNOMIAL DEGREE", "THREAD MODEL",
    "PLATFORM NUMBER", "DEVICE NUMBER", "LAMBDA", "DISCRETIZATION", "LINEAR SOLVER",
    "LINEAR SOLVER STOPPING CRITERION", "PRECONDITIONER", "MULTIGRID COARSENING",
    "MULTIGRID SMOOTHER", "MULTIGRID CHEBYSHEV DEGREE", "PARALMOND CYCLE", "PARALMOND STRENGTH",
    "PARALMOND AGGREGATION", "PARALMOND SMOOTHER", "PARALMOND CHEBYSHEV DEGREE", "OUTPUT TO FILE",
    "OUTPUT FILE NAME", "VERBOSE",
    // additions
    "MULTIGRID DEGREES", "PRECONDITIONER PRECISION", "FINE SMOOTHER", "MESH JITTER",
    "MESH JITTER SEED", "LAMBDA FIELD", "LAMBDA SEED", "RHS FIELD", "RHS SEED", "RHS SOURCES",
    "SOLVER TOLERANCE", "MAXIMUM ITERATIONS", "SMOOTHER TRAINING PAIRS",
    "LEARNED SMOOTHER STEPS", "OPERATOR PRECISION", "INITIAL GUESS STRATEGY",
    "INITIAL GUESS HISTORY SPACE DIMENSION", "INITIAL GUESS EXTRAP DEGREE", "INITIAL GUESS EXTRAP COEFFS METHOD"};

int Settings::parse(const std::string& text) {
  kv.clear();
  std::istringstream in(text);
  std::string line, key;
  bool haveKey = false;
  while (std::getline(in, line)) {
    auto h = line.find('#');
    if (h != std::string::npos) line = line.substr(0, h);
    line = trim(line);
    if (line.empty()) continue;
    if (line[0] == '[') {
      auto e = line.find(']');
      if (e == std::string::npos) return set_error(LPG_ERR_SETTINGS, "malformed settings line: " + line);
      key = trim(line.substr(1, e - 1));
      bool known = false;
      for (const char* k : kKnownKeys) known |= (key == k);
      if (!known) return set_error(LPG_ERR_SETTINGS, "unknown setting [" + key + "]");
      haveKey = true;
    } else if (haveKey) {
      kv[key] = line;
      haveKey = false;
    }
  }
  return LPG_OK;
}

std::string Settings::get(const std::string& k, const std::string& def) const {
  auto it = kv.find(k);
  return it == kv.end() ? def : it->second;
}
int Settings::geti(const std::string& k, int def) const {
  auto it = kv.find(k);
  return it == kv.end() ? def : std::atoi(it->second.c_str());
}
double Settings::getd(const std::string& k, double def) const {
  auto it = kv.find(k);
  return it == kv.end() ? def : std::atof(it->second.c_str());
}

// ---------------------------------------------------------------- device buffers
static std::atomic<int64_t> g_device_bytes{0};
int64_t device_bytes_in_use() { return g_device_bytes.load(); }

template <typename T>
int DevBuf<T>::alloc(int64_t count) {
  release();
  if (count <= 0) return LPG_OK;
  void* ptr = nullptr;
  cudaError_t e = cudaMalloc(&ptr, sizeof(T) * (size_t)count);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(LPG_ERR_ALLOC, std::string("cudaMalloc of ") + std::to_string(sizeof(T) * count) +
                                        " bytes failed: " + cudaGetErrorString(e));
  }
  p = (T*)ptr;
  n = count;
  g_device_bytes += bytes();
  return LPG_OK;
}
template <typename T>
int DevBuf<T>::upload(const T* host, int64_t count, cudaStream_t s) {
  if (count > n) return set_error(LPG_ERR_INVALID, "upload larger than buffer");
  if (count <= 0) return LPG_OK;
  cudaError_t e = cudaMemcpyAsync(p, host, sizeof(T) * count, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(LPG_ERR_CUDA, std::string("upload: ") + cudaGetErrorString(e));
  return LPG_OK;
}
template <typename T>
int DevBuf<T>::download(T* host, int64_t count, cudaStream_t s) const {
  if (count > n) return set_error(LPG_ERR_INVALID, "download larger than buffer");
  if (count <= 0) return LPG_OK;
  cudaError_t e = cudaMemcpyAsync(host, p, sizeof(T) * count, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return set_error(LPG_ERR_CUDA, std::string("download: ") + cudaGetErrorString(e));
  return LPG_OK;
}
template <typename T>
void DevBuf<T>::release() {
  if (p) {
    cudaFree(p);
    g_device_bytes -= bytes();
  }
  p = nullptr;
  n = 0;
}
template struct DevBuf<double>;
template struct DevBuf<float>;
template struct DevBuf<int32_t>;
template struct DevBuf<int64_t>;
template struct DevBuf<__nv_bfloat16>;
template struct DevBuf<float2>;

// ---------------------------------------------------------------- hashing
uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
// Uniform [0,1) keyed by (seed, stream, key): independent of element order and partition.
double hash_u01(uint64_t seed, uint64_t stream, uint64_t key) {
  const uint64_t h = splitmix64(splitmix64(seed ^ (stream << 56)) + key);
  return (double)(h >> 11) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------- GLL basis
// Legendre P_N and derivative by the three-term recurrence.
static void legendre(int N, double x, double& P, double& dP) {
  double p0 = 1, p1 = x;
  if (N == 0) { P = 1; dP = 0; return; }
  for (int k = 2; k <= N; ++k) {
    const double p2 = ((2 * k - 1) * x * p1 - (k - 1) * p0) / k;
    p0 = p1;
    p1 = p2;
  }
  P = p1;
  dP = (std::fabs(x) < 1.0) ? N * (x * p1 - p0) / (x * x - 1) : 0.5 * x * N * (N + 1) * std::pow(x, N);
}

// GLL nodes: x = +-1 and the roots of P_N'(x), by Newton's method from
// Chebyshev-Gauss-Lobatto guesses with P_N'' from the Legendre equation
// (1-x^2) P'' = 2x P' - N(N+1) P. Weights 2 / (N(N+1) P_N(x)^2).
void gll_nodes_weights(int N, std::vector<double>& x, std::vector<double>& w) {
  x.assign(N + 1, 0.0);
  w.assign(N + 1, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 1; i < N; ++i) {
    double xi = -std::cos(pi * i / N);
    for (int it = 0; it < 100; ++it) {
      double P, dP;
      legendre(N, xi, P, dP);
      const double d2P = (2 * xi * dP - N * (N + 1) * P) / (1 - xi * xi);
      const double dx = dP / d2P;
      xi -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    x[i] = xi;
  }
  x[0] = -1.0;
  x[N] = 1.0;
  // symmetrise (nodes are symmetric about 0)
  for (int i = 0; i <= N / 2; ++i) {
    const double v = 0.5 * (x[N - i] - x[i]);
    x[i] = -v;
    x[N - i] = v;
  }
  if (N % 2 == 0) x[N / 2] = 0.0;
  for (int i = 0; i <= N; ++i) {
    double P, dP;
    legendre(N, x[i], P, dP);
    w[i] = 2.0 / (N * (N + 1) * P * P);
  }
}

// D[i*Nq+j] = l_j'(x_i) by the barycentric formula.
void gll_derivative(int N, const std::vector<double>& x, std::vector<double>& D) {
  const int Nq = N + 1;
  std::vector<double> bw(Nq, 1.0);
  for (int j = 0; j < Nq; ++j)
    for (int k = 0; k < Nq; ++k)
      if (k != j) bw[j] /= (x[j] - x[k]);
  D.assign(Nq * Nq, 0.0);
  for (int i = 0; i < Nq; ++i) {
    double diag = 0;
    for (int j = 0; j < Nq; ++j) {
      if (i == j) continue;
      const double v = (bw[j] / bw[i]) / (x[i] - x[j]);
      D[i * Nq + j] = v;
      diag -= v;
    }
    D[i * Nq + i] = diag;
  }
}

void gll_interpolation(int Nc, int Nf, std::vector<double>& P) {
  std::vector<double> xc, wc, xf, wf;
  gll_nodes_weights(Nc, xc, wc);
  gll_nodes_weights(Nf, xf, wf);
  const int Nqc = Nc + 1, Nqf = Nf + 1;
  P.assign(Nqf * Nqc, 0.0);
  for (int i = 0; i < Nqf; ++i)
    for (int m = 0; m < Nqc; ++m) {
      double l = 1;
      for (int k = 0; k < Nqc; ++k)
        if (k != m) l *= (xf[i] - xc[k]) / (xc[m] - xc[k]);
      P[i * Nqc + m] = l;
    }
}

// Spectral radius of an upper-Hessenberg matrix (column-major, as the Arnoldi H of
// ellipticPreconMultiGridLevel.cpp:441-458) by implicit double-shift QR sweeps.
double hessenberg_spectral_radius(int n, const std::vector<double>& Hc) {
  std::vector<double> A(n * n, 0.0), wr(n, 0.0), wi(n, 0.0);
  auto a = [&](int i, int j) -> double& { return A[i * n + j]; };
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) a(i, j) = (j >= i - 1) ? Hc[i + j * n] : 0.0;
  int hi = n - 1, iter = 0;
  const double eps = 2.220446049250313e-16;
  while (hi >= 0) {
    if (hi == 0) { wr[0] = a(0, 0); hi--; continue; }
    int l = hi;
    while (l > 0) {
      double sc = std::fabs(a(l - 1, l - 1)) + std::fabs(a(l, l));
      if (sc == 0.0) sc = 1.0;
      if (std::fabs(a(l, l - 1)) <= eps * sc) { a(l, l - 1) = 0.0; break; }
      l--;
    }
    if (l == hi) { wr[hi] = a(hi, hi); hi--; iter = 0; continue; }
    if (l == hi - 1) {
      const double aa = a(hi - 1, hi - 1), b = a(hi - 1, hi), c = a(hi, hi - 1), d = a(hi, hi);
      const double p = 0.5 * (aa - d), disc = p * p + b * c, m = 0.5 * (aa + d);
      if (disc >= 0) {
        const double sq = std::sqrt(disc);
        const double z = p + (p >= 0 ? sq : -sq);
        wr[hi - 1] = d + z;
        wr[hi] = (z != 0.0) ? d - b * c / z : d;
      } else {
        const double sq = std::sqrt(-disc);
        wr[hi - 1] = wr[hi] = m;
        wi[hi - 1] = sq;
        wi[hi] = -sq;
      }
      hi -= 2;
      iter = 0;
      continue;
    }
    if (iter > 300) {
      for (int i = l; i <= hi; ++i) wr[i] = a(i, i);
      hi = l - 1;
      iter = 0;
      continue;
    }
    double s, t;
    if (iter > 0 && iter % 11 == 0) {
      const double e = std::fabs(a(hi, hi - 1)) + std::fabs(a(hi - 1, hi - 2));
      s = 1.5 * e;
      t = e * e;
    } else {
      s = a(hi - 1, hi - 1) + a(hi, hi);
      t = a(hi - 1, hi - 1) * a(hi, hi) - a(hi - 1, hi) * a(hi, hi - 1);
    }
    double x = a(l, l) * a(l, l) + a(l, l + 1) * a(l + 1, l) - s * a(l, l) + t;
    double y = a(l + 1, l) * (a(l, l) + a(l + 1, l + 1) - s);
    double z = a(l + 1, l) * a(l + 2, l + 1);
    for (int k = l; k <= hi - 2; ++k) {
      const double nv = std::sqrt(x * x + y * y + z * z);
      if (nv != 0.0) {
        const double alpha = (x >= 0) ? -nv : nv;
        const double u0 = x - alpha, u1 = y, u2 = z;
        const double uu = u0 * u0 + u1 * u1 + u2 * u2;
        if (uu != 0.0) {
          const double beta = 2.0 / uu;
          const int c0 = (k > l) ? k - 1 : l;
          for (int j = c0; j <= hi; ++j) {
            const double dd = beta * (u0 * a(k, j) + u1 * a(k + 1, j) + u2 * a(k + 2, j));
            a(k, j) -= dd * u0; a(k + 1, j) -= dd * u1; a(k + 2, j) -= dd * u2;
          }
          const int r1 = std::min(k + 3, hi);
          for (int i = l; i <= r1; ++i) {
            const double dd = beta * (u0 * a(i, k) + u1 * a(i, k + 1) + u2 * a(i, k + 2));
            a(i, k) -= dd * u0; a(i, k + 1) -= dd * u1; a(i, k + 2) -= dd * u2;
          }
        }
      }
      x = a(k + 1, k);
      y = a(k + 2, k);
      z = (k < hi - 2) ? a(k + 3, k) : 0.0;
    }
    {
      const int k = hi - 1;
      const double r = std::hypot(x, y);
      if (r != 0.0) {
        const double c = x / r, sn = y / r;
        const int c0 = (k > l) ? k - 1 : l;
        for (int j = c0; j <= hi; ++j) {
          const double a1 = a(k, j), a2 = a(k + 1, j);
          a(k, j) = c * a1 + sn * a2;
          a(k + 1, j) = -sn * a1 + c * a2;
        }
        for (int i = l; i <= hi; ++i) {
          const double a1 = a(i, k), a2 = a(i, k + 1);
          a(i, k) = c * a1 + sn * a2;
          a(i, k + 1) = -sn * a1 + c * a2;
        }
      }
    }
    iter++;
  }
  double rho = 0;
  for (int i = 0; i < n; ++i) rho = std::max(rho, std::sqrt(wr[i] * wr[i] + wi[i] * wi[i]));
  return rho;
}

// ---------------------------------------------------------------- platform
int Platform::init() {
  // A blocking stream: work queued by callers on the legacy default stream is ordered
  // before this object's kernels and vice versa.
  LPG_CUDA_TRY(cudaStreamCreate(&stream));
  int rc = partials.alloc(kReducePartials);
  if (rc) return rc;
  rc = scalars.alloc(16);
  if (rc) return rc;
  LPG_CUDA_TRY(cudaMallocHost(&hostScalars, 16 * sizeof(double)));
  return LPG_OK;
}

Platform::~Platform() {
  if (hostScalars) cudaFreeHost(hostScalars);
  if (stream) cudaStreamDestroy(stream);
}

int Platform::dot(int64_t n, const double* x, const double* y, double& out) {
  int rc = lpg::dot(n, x, y, scalars.p, partials.p, stream);
  if (rc) return rc;
  LPG_CUDA_TRY(cudaMemcpyAsync(hostScalars, scalars.p, sizeof(double), cudaMemcpyDeviceToHost, stream));
  LPG_CUDA_TRY(cudaStreamSynchronize(stream));
  out = hostScalars[0];
  return LPG_OK;
}

int Platform::sum(int64_t n, const double* x, double& out) {
  int rc = lpg::sum(n, x, scalars.p, partials.p, stream);
  if (rc) return rc;
  LPG_CUDA_TRY(cudaMemcpyAsync(hostScalars, scalars.p, sizeof(double), cudaMemcpyDeviceToHost, stream));
  LPG_CUDA_TRY(cudaStreamSynchronize(stream));
  out = hostScalars[0];
  return LPG_OK;
}

}  // namespace lpg
