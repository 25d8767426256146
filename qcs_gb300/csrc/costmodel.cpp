// costmodel.cpp -- learned fusion cost model, host side (placeholder).
