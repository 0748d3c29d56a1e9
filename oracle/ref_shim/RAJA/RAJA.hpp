// Empty stand-in: the element kernels compiled here use no RAJA symbol.
#pragma once
