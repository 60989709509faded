// Parallel text output for the driver's outfiles (restart and movie files of src/md.cpp:526-546,
// 647-678): lines formatted on the host's cores, byte-identical to one sequential iostream pass.
#pragma once
#include <algorithm>
#include <ostream>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

// Lines [0, n) formatted by line(os, i) on the host's cores, in chunks written into strings and
// appended to out in order.  Each chunk's stream starts in out's state as it would be at the
// chunk's first line: out's current precision and width for the first chunk, and the precision
// and pending width the lines leave behind (`later_prec`, `later_width`) for the others; lines end
// with an unformatted put('\n'), which, like endl, leaves a pending width alone.  So the bytes are
// those of one sequential pass.
template <class Line>
inline void write_lines(std::ostream& out, long n, std::streamsize later_prec, std::streamsize later_width, Line line) {
  const long min_chunk = 4096;
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const long chunks = std::max(1L, std::min<long>((long)std::min(hw, 16u), n / min_chunk));
  std::vector<std::string> text((size_t)chunks);
  auto run = [&](long c) {
    std::ostringstream os;
    os.flags(out.flags());
    os.fill(out.fill());
    os.precision(c == 0 ? out.precision() : later_prec);
    os.width(c == 0 ? out.width() : later_width);
    const long i0 = n * c / chunks, i1 = n * (c + 1) / chunks;
    for (long i = i0; i < i1; i++) line(os, i);
    text[(size_t)c] = os.str();
  };
  std::vector<std::thread> pool;
  for (long c = 1; c < chunks; c++) pool.emplace_back(run, c);
  run(0);
  for (auto& t : pool) t.join();
  const std::streamsize w = out.width();
  out.width(0);
  for (const auto& t : text) out << t;
  out.width(n > 0 ? later_width : w);
  if (n > 0) out.precision(later_prec);
  out.flush();
}
