// cos / sin (2 pi e / R) for the in-register DFT twiddles, e < R, as switch
// functions that fold to immediates once e is a compile-time constant.
// Generated (correctly rounded) by gato_gb300/csrc/gen_twiddles.py.
#pragma once

namespace gato {

template <int R> struct TwC;
template <> struct TwC<4> {
  __host__ __device__ static constexpr double c(int e) {
    switch (e) {
      case 0: return 1.0;
      case 1: return 0.0;
      case 2: return -1.0;
      case 3: return 0.0;
      default: return 0.0;
    }
  }
  __host__ __device__ static constexpr double s(int e) {
    switch (e) {
      case 0: return 0.0;
      case 1: return 1.0;
      case 2: return 0.0;
      case 3: return -1.0;
      default: return 0.0;
    }
  }
};
template <> struct TwC<6> {
  __host__ __device__ static constexpr double c(int e) {
    switch (e) {
      case 0: return 1.0;
      case 1: return 0.5;
      case 2: return -0.5;
      case 3: return -1.0;
      case 4: return -0.5;
      case 5: return 0.5;
      default: return 0.0;
    }
  }
  __host__ __device__ static constexpr double s(int e) {
    switch (e) {
      case 0: return 0.0;
      case 1: return 0.8660254037844386;
      case 2: return 0.8660254037844386;
      case 3: return 0.0;
      case 4: return -0.8660254037844386;
      case 5: return -0.8660254037844386;
      default: return 0.0;
    }
  }
};
template <> struct TwC<8> {
  __host__ __device__ static constexpr double c(int e) {
    switch (e) {
      case 0: return 1.0;
      case 1: return 0.7071067811865476;
      case 2: return 0.0;
      case 3: return -0.7071067811865476;
      case 4: return -1.0;
      case 5: return -0.7071067811865476;
      case 6: return 0.0;
      case 7: return 0.7071067811865476;
      default: return 0.0;
    }
  }
  __host__ __device__ static constexpr double s(int e) {
    switch (e) {
      case 0: return 0.0;
      case 1: return 0.7071067811865476;
      case 2: return 1.0;
      case 3: return 0.7071067811865476;
      case 4: return 0.0;
      case 5: return -0.7071067811865476;
      case 6: return -1.0;
      case 7: return -0.7071067811865476;
      default: return 0.0;
    }
  }
};
template <> struct TwC<10> {
  __host__ __device__ static constexpr double c(int e) {
    switch (e) {
      case 0: return 1.0;
      case 1: return 0.8090169943749475;
      case 2: return 0.30901699437494745;
      case 3: return -0.30901699437494745;
      case 4: return -0.8090169943749475;
      case 5: return -1.0;
      case 6: return -0.8090169943749475;
      case 7: return -0.30901699437494745;
      case 8: return 0.30901699437494745;
      case 9: return 0.8090169943749475;
      default: return 0.0;
    }
  }
  __host__ __device__ static constexpr double s(int e) {
    switch (e) {
      case 0: return 0.0;
      case 1: return 0.5877852522924731;
      case 2: return 0.9510565162951535;
      case 3: return 0.9510565162951535;
      case 4: return 0.5877852522924731;
      case 5: return 0.0;
      case 6: return -0.5877852522924731;
      case 7: return -0.9510565162951535;
      case 8: return -0.9510565162951535;
      case 9: return -0.5877852522924731;
      default: return 0.0;
    }
  }
};
template <> struct TwC<12> {
  __host__ __device__ static constexpr double c(int e) {
    switch (e) {
      case 0: return 1.0;
      case 1: return 0.8660254037844386;
      case 2: return 0.5;
      case 3: return 0.0;
      case 4: return -0.5;
      case 5: return -0.8660254037844386;
      case 6: return -1.0;
      case 7: return -0.8660254037844386;
      case 8: return -0.5;
      case 9: return 0.0;
      case 10: return 0.5;
      case 11: return 0.8660254037844386;
      default: return 0.0;
    }
  }
  __host__ __device__ static constexpr double s(int e) {
    switch (e) {
      case 0: return 0.0;
      case 1: return 0.5;
      case 2: return 0.8660254037844386;
      case 3: return 1.0;
      case 4: return 0.8660254037844386;
      case 5: return 0.5;
      case 6: return 0.0;
      case 7: return -0.5;
      case 8: return -0.8660254037844386;
      case 9: return -1.0;
      case 10: return -0.8660254037844386;
      case 11: return -0.5;
      default: return 0.0;
    }
  }
};
template <> struct TwC<14> {
  __host__ __device__ static constexpr double c(int e) {
    switch (e) {
      case 0: return 1.0;
      case 1: return 0.9009688679024191;
      case 2: return 0.6234898018587335;
      case 3: return 0.2225209339563144;
      case 4: return -0.2225209339563144;
      case 5: return -0.6234898018587335;
      case 6: return -0.9009688679024191;
      case 7: return -1.0;
      case 8: return -0.9009688679024191;
      case 9: return -0.6234898018587335;
      case 10: return -0.2225209339563144;
      case 11: return 0.2225209339563144;
      case 12: return 0.6234898018587335;
      case 13: return 0.9009688679024191;
      default: return 0.0;
    }
  }
  __host__ __device__ static constexpr double s(int e) {
    switch (e) {
      case 0: return 0.0;
      case 1: return 0.4338837391175581;
      case 2: return 0.7818314824680298;
      case 3: return 0.9749279121818236;
      case 4: return 0.9749279121818236;
      case 5: return 0.7818314824680298;
      case 6: return 0.4338837391175581;
      case 7: return 0.0;
      case 8: return -0.4338837391175581;
      case 9: return -0.7818314824680298;
      case 10: return -0.9749279121818236;
      case 11: return -0.9749279121818236;
      case 12: return -0.7818314824680298;
      case 13: return -0.4338837391175581;
      default: return 0.0;
    }
  }
};
template <> struct TwC<16> {
  __host__ __device__ static constexpr double c(int e) {
    switch (e) {
      case 0: return 1.0;
      case 1: return 0.9238795325112867;
      case 2: return 0.7071067811865476;
      case 3: return 0.3826834323650898;
      case 4: return 0.0;
      case 5: return -0.3826834323650898;
      case 6: return -0.7071067811865476;
      case 7: return -0.9238795325112867;
      case 8: return -1.0;
      case 9: return -0.9238795325112867;
      case 10: return -0.7071067811865476;
      case 11: return -0.3826834323650898;
      case 12: return 0.0;
      case 13: return 0.3826834323650898;
      case 14: return 0.7071067811865476;
      case 15: return 0.9238795325112867;
      default: return 0.0;
    }
  }
  __host__ __device__ static constexpr double s(int e) {
    switch (e) {
      case 0: return 0.0;
      case 1: return 0.3826834323650898;
      case 2: return 0.7071067811865476;
      case 3: return 0.9238795325112867;
      case 4: return 1.0;
      case 5: return 0.9238795325112867;
      case 6: return 0.7071067811865476;
      case 7: return 0.3826834323650898;
      case 8: return 0.0;
      case 9: return -0.3826834323650898;
      case 10: return -0.7071067811865476;
      case 11: return -0.9238795325112867;
      case 12: return -1.0;
      case 13: return -0.9238795325112867;
      case 14: return -0.7071067811865476;
      case 15: return -0.3826834323650898;
      default: return 0.0;
    }
  }
};
template <> struct TwC<20> {
  __host__ __device__ static constexpr double c(int e) {
    switch (e) {
      case 0: return 1.0;
      case 1: return 0.9510565162951535;
      case 2: return 0.8090169943749475;
      case 3: return 0.5877852522924731;
      case 4: return 0.30901699437494745;
      case 5: return 0.0;
      case 6: return -0.30901699437494745;
      case 7: return -0.5877852522924731;
      case 8: return -0.8090169943749475;
      case 9: return -0.9510565162951535;
      case 10: return -1.0;
      case 11: return -0.9510565162951535;
      case 12: return -0.8090169943749475;
      case 13: return -0.5877852522924731;
      case 14: return -0.30901699437494745;
      case 15: return 0.0;
      case 16: return 0.30901699437494745;
      case 17: return 0.5877852522924731;
      case 18: return 0.8090169943749475;
      case 19: return 0.9510565162951535;
      default: return 0.0;
    }
  }
  __host__ __device__ static constexpr double s(int e) {
    switch (e) {
      case 0: return 0.0;
      case 1: return 0.30901699437494745;
      case 2: return 0.5877852522924731;
      case 3: return 0.8090169943749475;
      case 4: return 0.9510565162951535;
      case 5: return 1.0;
      case 6: return 0.9510565162951535;
      case 7: return 0.8090169943749475;
      case 8: return 0.5877852522924731;
      case 9: return 0.30901699437494745;
      case 10: return 0.0;
      case 11: return -0.30901699437494745;
      case 12: return -0.5877852522924731;
      case 13: return -0.8090169943749475;
      case 14: return -0.9510565162951535;
      case 15: return -1.0;
      case 16: return -0.9510565162951535;
      case 17: return -0.8090169943749475;
      case 18: return -0.5877852522924731;
      case 19: return -0.30901699437494745;
      default: return 0.0;
    }
  }
};
template <> struct TwC<24> {
  __host__ __device__ static constexpr double c(int e) {
    switch (e) {
      case 0: return 1.0;
      case 1: return 0.9659258262890683;
      case 2: return 0.8660254037844386;
      case 3: return 0.7071067811865476;
      case 4: return 0.5;
      case 5: return 0.25881904510252074;
      case 6: return 0.0;
      case 7: return -0.25881904510252074;
      case 8: return -0.5;
      case 9: return -0.7071067811865476;
      case 10: return -0.8660254037844386;
      case 11: return -0.9659258262890683;
      case 12: return -1.0;
      case 13: return -0.9659258262890683;
      case 14: return -0.8660254037844386;
      case 15: return -0.7071067811865476;
      case 16: return -0.5;
      case 17: return -0.25881904510252074;
      case 18: return 0.0;
      case 19: return 0.25881904510252074;
      case 20: return 0.5;
      case 21: return 0.7071067811865476;
      case 22: return 0.8660254037844386;
      case 23: return 0.9659258262890683;
      default: return 0.0;
    }
  }
  __host__ __device__ static constexpr double s(int e) {
    switch (e) {
      case 0: return 0.0;
      case 1: return 0.25881904510252074;
      case 2: return 0.5;
      case 3: return 0.7071067811865476;
      case 4: return 0.8660254037844386;
      case 5: return 0.9659258262890683;
      case 6: return 1.0;
      case 7: return 0.9659258262890683;
      case 8: return 0.8660254037844386;
      case 9: return 0.7071067811865476;
      case 10: return 0.5;
      case 11: return 0.25881904510252074;
      case 12: return 0.0;
      case 13: return -0.25881904510252074;
      case 14: return -0.5;
      case 15: return -0.7071067811865476;
      case 16: return -0.8660254037844386;
      case 17: return -0.9659258262890683;
      case 18: return -1.0;
      case 19: return -0.9659258262890683;
      case 20: return -0.8660254037844386;
      case 21: return -0.7071067811865476;
      case 22: return -0.5;
      case 23: return -0.25881904510252074;
      default: return 0.0;
    }
  }
};

}  // namespace gato
