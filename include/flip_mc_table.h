/*
 * flip_mc_table.h — marching-cubes case table shared by the CUDA mesher and
 * the CPU oracle.
 *
 * Cell corners c = 0..7 sit at offsets (dx,dy,dz) = FLIP_MC_CORNER[c]; a
 * corner is "inside" when its field value is below the iso level, and the
 * case index has bit c set for inside corners. Edge e joins corners
 * FLIP_MC_EDGE_ENDS[e]; an edge is cut when exactly one of its corners is
 * inside, so the cut-edge mask of a case follows from the corners and is
 * not tabulated.
 *
 * FLIP_MC_TRIS[case] lists the triangles of the case as cut-edge numbers,
 * one hex digit per edge, three digits per triangle. It is the public-domain
 * marching-cubes triangulation published by Paul Bourke (after Cory Gene
 * Bloyd), the same one the reference's isosurface extractor uses
 * (src/rchandra/CIsoSurface.cpp). It has to be identical, not merely
 * equivalent: triangle order and winding decide the face list, the order of
 * the per-vertex normal sums and the smoothing neighbour lists.
 */
#ifndef FLIP_MC_TABLE_H
#define FLIP_MC_TABLE_H

/* corner offsets (dx, dy, dz) */
static const unsigned char FLIP_MC_CORNER[8][3] = {
    {0, 0, 0}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0},
    {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {1, 0, 1}};

/* corners joined by each edge */
static const unsigned char FLIP_MC_EDGE_ENDS[12][2] = {
    {0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
    {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

/* Each edge as (base-node offset dx, dy, dz, axis 0=x 1=y 2=z): the global
 * edge it names is the axis-aligned edge leaving that node in +axis. */
static const unsigned char FLIP_MC_EDGE_NODE[12][4] = {
    {0, 0, 0, 1}, {0, 1, 0, 0}, {1, 0, 0, 1}, {0, 0, 0, 0},
    {0, 0, 1, 1}, {0, 1, 1, 0}, {1, 0, 1, 1}, {0, 0, 1, 0},
    {0, 0, 0, 2}, {0, 1, 0, 2}, {1, 1, 0, 2}, {1, 0, 0, 2}};

/* triangles per case, three edge digits each */
static const char *const FLIP_MC_TRIS[256] = {
    "", "083", "019", "183981", "12a", "08312a", "92a029", "2832a8a98",
    "3b2", "0b28b0", "19023b", "1b219b98b", "3a1ba3", "0a108a8ba", "3903b9ba9", "98aa8b",
    "478", "430734", "019847", "419471731", "12a847", "34730412a", "92a902847", "2a9297273794",
    "8473b2", "b47b24204", "90184723b", "47b94b9b2921", "3a13ba784", "1ba14b1047b4", "47890b9bab03", "47b4b99ba",
    "954", "954083", "054150", "854835315", "12a954", "30812a495", "52a542402", "2a5325354348",
    "95423b", "0b208b495", "05401523b", "21525828b485", "a3ba13954", "4950818a18ba", "54050b5bab03", "54858aa8b",
    "978579", "930953573", "078017157", "153357", "978957a12", "a12950530573", "802825857a52", "2a5253357",
    "7957893b2", "95797292027b", "23b018178157", "b21b17715", "958857a13a3b", "5705097b010aba0", "ba0b03a50807570", "ba57b5",
    "a65", "0835a6", "9015a6", "1831985a6", "165261", "165126308", "965906026", "598582526328",
    "23ba65", "b08b20a65", "01923b5a6", "5a61929b298b", "63b653513", "08b0b50515b6", "3b6036065059", "65969bb98",
    "5a6478", "43047365a", "1905a6847", "a65197173794", "612651478", "125526304347", "847905065026", "739794329596269",
    "3b2784a65", "5a647242027b", "01947823b5a6", "9219b294b7b45a6", "8473b53515b6", "51b5b610b7b404b", "059065036b63847", "65969b4797b9",
    "a4964a", "4a649a083", "a01a60640", "83181686461a", "149124264", "308129249264", "024426", "832824426",
    "a49a64b23", "08228b49a4a6", "3b201606461a", "64161a48121b8b1", "964936913b63", "8b1810b61914641", "3b6360064", "648b68",
    "7a678a89a", "0730a709a67a", "a671a7178180", "a67a71173", "126168189867", "269291679093739", "780706602", "732672",
    "23ba68a89867", "20727b09767a9a7", "1801781a767a23b", "b21b17a61671", "896867916b63136", "091b67", "7807063b0b60", "7b6",
    "76b", "308b76", "019b76", "819831b76", "a126b7", "12a3086b7", "2902a96b7", "6b72a3a83a98",
    "723627", "708760620", "276237019", "162186198876", "a76a17137", "a7617a187108", "03707a0a96a7", "76a7a88a9",
    "684b86", "36b306046", "86b846901", "946963931b36", "6846b82a1", "12a30b06b046", "4b846b0292a9", "a93a32943b36463",
    "823842462", "042462", "190234246438", "194142246", "8138618466a1", "a10a06604", "4634386a3039a93", "a946a4",
    "49576b", "083495b76", "50154076b", "b76834354315", "954a1276b", "6b712a083495", "76b54a42a402", "348354325a52b76",
    "723762549", "954086062687", "362376150540", "628687218485158", "954a16176137", "16a176107870954", "40a4a503a6a737a", "76a7a854a48a",
    "6956b9b89", "36b063056095", "0b805b01556b", "6b3635531", "12a95b9b8b56", "0b306b09656912a", "b85b56805a52025", "6b36352a3a53",
    "589528562382", "956960062", "158180568382628", "156216", "13616a386569896", "a10a06950560", "03856a", "a56",
    "b5a75b", "b5ab75830", "5b75ab190", "a75ab7981831", "b12b71751", "08312717572b", "9759279022b7", "75272b592328982",
    "25a235375", "820852875a25", "9015a35373a2", "982921872a25752", "135375", "087071175", "903935537", "987597",
    "5845a8ab8", "5045b05abb30", "01984a8aba45", "ab4a45b34941314", "2512852b8458", "04b0b345b2b151b", "0250592b5458b85", "9452b3",
    "25a352345384", "5a2524420", "3a235a385458019", "5a2524192942", "845853351", "045105", "845853905035", "945",
    "4b749b9ab", "0834979b79ab", "1ab1b414074b", "3143481a474bab4", "4b79b492b912", "9749b791b2b1083", "b74b42240", "b74b42834324",
    "29a279237749", "9a7974a27870207", "37a3a274a1a040a", "1a2874", "491417713", "491417081871", "403743", "487",
    "9a8ab8", "30939bb9a", "01a0a88ab", "31ab3a", "12b1b99b8", "30939b1292b9", "02b80b", "32b",
    "23828aa89", "9a2092", "23828a0181a8", "1a2", "138918", "091", "038", "",
};

/* Decode FLIP_MC_TRIS into tri[256][16] (edge numbers, -1 terminated) and
 * count[256] (triangles per case). */
static inline void flip_mc_decode(signed char tri[256][16], unsigned char count[256]) {
  for (int c = 0; c < 256; c++) {
    int m = 0;
    for (const char *s = FLIP_MC_TRIS[c]; *s; s++, m++)
      tri[c][m] = (signed char)(*s <= '9' ? *s - '0' : *s - 'a' + 10);
    count[c] = (unsigned char)(m / 3);
    for (; m < 16; m++) tri[c][m] = -1;
  }
}

#endif
