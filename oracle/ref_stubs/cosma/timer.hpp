// Stand-in for the reference's timer header (unused on the CPU path).
#pragma once
