// Board files and the base81 codec (host side of the CLI).
//
// File format (main.cu:49-67, README.md:27-41): a line holding the board
// count n, then n lines whose first 16 characters encode one board each.
// Codec (test.cpp:7-19; to_board.cpp:15-39 decodes): character i covers
// squares 4i..4i+3; square j of the group adds w_j for the side to move and
// 2*w_j for the other side, w = {1, 3, 9, 32}, plus 33.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gpo_host {

struct Board {
  uint64_t p, o;  // side to move, other side
  bool operator<(const Board& b) const { return p != b.p ? p < b.p : o < b.o; }
  bool operator==(const Board& b) const { return p == b.p && o == b.o; }
};

void encode(uint64_t p, uint64_t o, char out[17]);
// Returns false on a character outside the codec's alphabet or a square
// claimed by both sides.
bool decode(const char* s, uint64_t& p, uint64_t& o);

// Reads a board file, then sorts and removes duplicates as the reference
// does before solving (main.cu:64-65).  On failure returns false and sets
// `err` ("Failed to load boards" for a short file, as main.cu:57-59).
bool load_boards(const std::string& path, std::vector<Board>& out, std::string& err);

// "<base81> <score>\n" per board, in the given order (main.cu:164-171).
bool write_results(const std::string& path, const std::vector<Board>& boards,
                   const std::vector<int8_t>& score, std::string& err);

// Think mode: "<base81> <score> <move>\n" per board (main.cu:114-117), the
// move as column letter + row digit, "ps" for a pass (main.cu:31-39).
bool write_think_results(const std::string& path, const std::vector<Board>& boards,
                         const std::vector<int8_t>& score, const std::vector<int8_t>& best,
                         std::string& err);
std::string move_string(int move);

bool write_boards(const std::string& path, const std::vector<Board>& boards, std::string& err);

}  // namespace gpo_host
